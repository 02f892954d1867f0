"""Python mirror of refeff's real-space FMS interface, bound to the C ABI of
include/refeff_fms.h (librefeff_fms.so, built for sm_103a).

Names follow the reference:
  fms_yprep_cluster        crates/refeff-core/src/fms/cluster.rs:10-195 (with sortat)
  fms_real_space_plan      crates/refeff-core/src/fms/driver.rs:105-140
  fms_real_space_spectrum  crates/refeff-core/src/fms/driver.rs:231-239
  complex_lu_solve_batched crates/refeff-linalg/src/lu.rs:385-490 (faer c32 LU factor + solve)
Errors raise FmsError carrying the library status code (the reference
returns Result<_, FmsError>).  There is no CPU fallback: if the CUDA library
cannot be loaded, or no GPU is present, the calls fail.
"""
from __future__ import annotations

import ctypes as C
import re
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import build as _build

FORM_FP64_LU = 0
FORM_FP32_REFINED = 1
FORM_BICGSTAB = 2

STATUS_NAMES = {
    0: "OK", 1: "InvalidArgument", 2: "EmptyCluster", 3: "PotentialOutOfRange", 4: "MissingRepresentativePotential",
    5: "InvalidAngularLimit", 6: "NonFiniteInput", 7: "NonFiniteCoordinate", 8: "ZeroRho", 9: "SingularMatrix",
    10: "NotConverged", 11: "DuplicateAbsorber", 12: "MissingCentralAtom", 13: "Unsupported", 14: "Cuda",
    15: "OutOfMemory", 16: "InvalidTolerance", 17: "InvalidClusterRadius", 18: "ScratchLimit",
    19: "IterativeSolverBreakdown", 20: "DebyeError",
}


class FmsError(RuntimeError):
    def __init__(self, code: int, message: str = ""):
        name = STATUS_NAMES.get(code, f"status {code}")
        super().__init__(f"{name}: {message}" if message else name)
        self.code = code
        self.name = name


_lib = None
_p = C.c_void_p
_i = C.c_int


class _PlanInput(C.Structure):
    _fields_ = [
        ("n_atoms", C.c_int), ("positions_xyz", _p), ("potentials", _p), ("spin_channels", C.c_int),
        ("spin_selector", C.c_int), ("lfms", C.c_int), ("minv", C.c_int), ("max_potential", C.c_int),
        ("global_lmax", C.c_int), ("raw_potential_lmax", _p), ("direct_cutoff", C.c_float),
        ("mean_square_displacements", _p), ("sig2g", C.c_float), ("convergence_tolerance", C.c_float),
        ("zero_tolerance", C.c_float),
    ]


class _EnergyPoints(C.Structure):
    _fields_ = [("n_energies", C.c_int), ("wave_numbers", _p), ("phase_shifts", _p)]


class _Tuning(C.Structure):
    _fields_ = [("streams", C.c_int), ("buckets", C.c_int), ("seconds_default", C.c_double),
                ("seconds_tuned", C.c_double), ("from_cache", C.c_int)]


class _Report(C.Structure):
    _fields_ = [("seconds", C.c_double), ("refinement_iterations", C.c_int), ("residual_max", C.c_double),
                ("energies_failed", C.c_int), ("fp64_fallbacks", C.c_int)]


def header_functions() -> list[str]:
    """Names of every function declared in include/refeff_fms.h."""
    text = (Path(__file__).resolve().parents[1] / "include" / "refeff_fms.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w ]*?[\s\*]+(refeff_\w+)\s*\(", text, flags=re.M)


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load librefeff_fms.so (building it with nvcc if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise FmsError(14, f"{path} is not built")
        _build.build()
    lib = C.CDLL(str(path))
    sig = {
        "refeff_fms_abi_version": ([], _i),
        "refeff_fms_kernel_launches": ([], C.c_ulonglong),
        "refeff_fms_context_set_option": ([_p, _i, C.c_longlong], _i),
        "refeff_fms_context_create": ([_i, _p], _i),
        "refeff_fms_context_destroy": ([_p], None),
        "refeff_fms_last_error": ([_p], C.c_char_p),
        "refeff_fms_yprep_cluster": ([_i, _i, _i, _p, _p, C.c_float, _i, _p, _p, _p], _i),
        "refeff_fms_real_space_plan_create": ([_p, _p, _p], _i),
        "refeff_fms_real_space_plan_create_full": ([_p, _p, _p], _i),
        "refeff_fms_real_space_spectrum_full": ([_p, _p, _p, _p, _p, _p, _p], _i),
        "refeff_fms_write_gg_slice_bin": ([C.c_char_p, _i, _i, _i, _p], _i),
        "refeff_fms_reciprocal_integrate": ([_p, _i, _i, _p, _p, _p, _i, _p, _p], _i),
        "refeff_fms_reciprocal_core_hole": ([_i, _p, _i, _i, _p, _p], _i),
        "refeff_ff2x_xanes_mu": ([_i, _i, _i, _i, _i, _i, _p, _p, _p, _p, _p, C.c_double, C.c_double, C.c_double,
                                  C.c_double, _p, _p, _p], _i),
        "refeff_ff2x_xanes_mu_thermal": ([_i, _i, _i, _i, _i, _i, _p, _p, _p, _p, _p, C.c_double, C.c_double,
                                          C.c_double, C.c_double, C.c_double, _p, _p, _p], _i),
        "refeff_ff2x_xscorr": ([_i, _i, _i, _i, _p, _p, _p, _p, C.c_double, C.c_double, _p], _i),
        "refeff_ff2x_lorentz_convolve": ([_i, _p, _p, C.c_double, _p], _i),
        "refeff_ff2x_debye_factor": ([_i, _p, C.c_double, _p, _p, _p], _i),
        "refeff_fms_write_gg_diag_bin": ([C.c_char_p, _i, _i, _i, _p], _i),
        "refeff_fms_real_space_plan_destroy": ([_p], None),
        "refeff_fms_plan_query": ([_p, _p, _p, _p, _p], _i),
        "refeff_fms_plan_set_batch": ([_p, _i], _i),
        "refeff_fms_plan_set_refinement": ([_p, _i, C.c_double], _i),
        "refeff_fms_plan_set_profiling": ([_p, _i], _i),
        "refeff_fms_plan_phase_times": ([_p, _p, _i], _i),
        "refeff_fms_real_space_spectrum": ([_p, _p, _i, _p, _p, _p], _i),
        "refeff_fms_real_space_spectrum_device": ([_p, _i, _p, _p, _i, _p, _p, _p], _i),
        "refeff_fms_gg_section": ([_p, _p, _i, _p], _i),
        "refeff_fms_plan_refinement_stats": ([_p, _i, _p, _p, _p], _i),
        "refeff_complex_lu_solve_batched": ([_p, _i, _i, _i, _p, _p, _p, _i, _p, _p], _i),
        "refeff_fms_run_dir": ([_p, C.c_char_p, _i, _p], _i),
        "refeff_fms_write_gg_dat": ([C.c_char_p, _i, _i, _p], _i),
        "refeff_fms_phase_bin_dims": ([C.c_char_p, _p, _p, _p, _p], _i),
        "refeff_fms_phase_bin_read": ([C.c_char_p, _p, _p, _p, _p], _i),
        "refeff_fms_transition_matrix": ([_i, _i, _i, _p, _i, _i, _i, _i, C.c_double, _p, _p, _p], _i),
        "refeff_fms_mkgtr_trace": ([_p, _i, _i, _i, _i, _i, _p, _p, _p, _p, _i, _p], _i),
        "refeff_fms_mkgtr_trace_device": ([_p, _i, _i, _i, _i, _i, _p, _p, _p, C.c_longlong, C.c_longlong, _p, _p,
                                           _p], _i),
        "refeff_fms_run_mkgtr_dir": ([_p, C.c_char_p, _p], _i),
        "refeff_fms_write_fms_bin": ([C.c_char_p, C.c_double, _i, _i, _i, _i, _i, _i, _p], _i),
        "refeff_fms_write_gtr_dat": ([C.c_char_p, _i, _p, _p], _i),
        "refeff_fms_real_space_spectrum_multi": ([_p, _i, _p, _p, _i, _p, _p, _p], _i),
        "refeff_fms_debye_sigma2_table": ([_p, _i, _i, _p, _p, _i, _p, C.c_double, C.c_double, C.c_double,
                                           C.c_float, _p, _p], _i),
        "refeff_fms_precond_model_create": ([_p, _i, _i, C.c_ulonglong, _p], _i),
        "refeff_fms_precond_model_create_kind": ([_p, _i, _i, _i, C.c_ulonglong, _p], _i),
        "refeff_fms_precond_model_destroy": ([_p], None),
        "refeff_fms_precond_model_query": ([_p, _p, _p, _p, _p], _i),
        "refeff_fms_precond_get_params": ([_p, _p], _i),
        "refeff_fms_precond_set_params": ([_p, _p], _i),
        "refeff_fms_precond_loss_grad": ([_p, _i, _p, _p, _p, _p], _i),
        "refeff_fms_precond_train": ([_p, _i, _p, _p, _i, _i, C.c_float, C.c_ulonglong, _p], _i),
        "refeff_fms_precond_predict": ([_p, _i, _p, _p], _i),
        "refeff_fms_plan_set_preconditioner": ([_p, _p], _i),
        "refeff_fms_plan_set_bicgstab": ([_p, _i, C.c_double, _i], _i),
        "refeff_fms_plan_bicgstab_stats": ([_p, _i, _p], _i),
        "refeff_fms_plan_precond_features": ([_p, _p, _p], _i),
        "refeff_fms_plan_inverse_diagonal": ([_p, _p, _i, _p, _p], _i),
        "refeff_fms_plan_inverse_block": ([_p, _p, _i, _p, _p], _i),
        "refeff_fms_geometry_from_feff_inp": ([C.c_char_p, _i, _p, _p, _p, _i, _p, _p], _i),
        "refeff_fms_autotune_multi": ([_p, _i, _p, _p, _i, _i, C.c_char_p, _p], _i),
        "refeff_fms_plan_set_tuning": ([_p, _i, _i], _i),
        "refeff_fms_plan_set_precond_window": ([_p, C.c_double, C.c_double], _i),
        "refeff_fms_plan_set_bicgstab_window": ([_p, C.c_double, C.c_double], _i),
        "refeff_fms_context_graph_stats": ([_p, _p, _p], _i),
        "refeff_fms_plan_bicgstab_lu_energies": ([_p, _i, _p], _i),
        "refeff_fms_plan_get_tuning": ([_p, _p, _p], _i),
        "refeff_fms_write_geom_dat": ([C.c_char_p, C.c_char_p], _i),
        "refeff_fms_feff_inp_last_error": ([], C.c_char_p),
        "refeff_ff2x_read_xsect_dat": ([C.c_char_p, C.c_double, _i, _i, _p, _p, _p, _p, _p, _p, _p], _i),
        "refeff_ff2x_xsect_last_error": ([], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_p)


def fms_yprep_cluster(positions, potentials, *, central_potential=0, max_potential=None, cluster_radius,
                      cluster_capacity=None):
    """FEFF yprep + sortat on the host library: absorber first, at the origin."""
    lib = load()
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
    pots = np.ascontiguousarray(potentials, dtype=np.int32)
    n = len(pots)
    maxp = int(pots.max()) if max_potential is None else int(max_potential)
    cap = n if cluster_capacity is None else int(cluster_capacity)
    out_pos = np.zeros_like(pos)
    out_pot = np.zeros_like(pots)
    cnt = np.zeros(1, np.int32)
    rc = lib.refeff_fms_yprep_cluster(int(central_potential), maxp, n, _ptr(pots), _ptr(pos), float(cluster_radius),
                                      cap, _ptr(out_pos), _ptr(out_pot), _ptr(cnt))
    if rc:
        raise FmsError(rc)
    return out_pos[: cnt[0]].copy(), out_pot[: cnt[0]].copy()


class Context:
    """One CUDA device, one stream (refeff_fms_context)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = _p()
        rc = self._lib.refeff_fms_context_create(int(device), C.byref(h))
        if rc:
            raise FmsError(rc, "cannot create a CUDA context (no GPU?)")
        self.handle = h

    OPT_TENSOR_CORES = 1
    OPT_DENSE_REFINEMENT = 2
    OPT_TC_WAIT_POLLS = 3
    OPT_PAIRED_BLOCKS = 4
    OPT_MULTI_STREAMS = 5
    OPT_DUAL_STREAMS = 6
    OPT_MULTI_GRAPH = 7
    OPT_BICG_TENSOR = 8
    OPT_RESIDUAL_TENSOR = 9

    def set_option(self, option: int, value: int):
        """Context option (applies to plans / dense solves started afterwards)."""
        self.check(self._lib.refeff_fms_context_set_option(self.handle, int(option), int(value)))

    def graph_stats(self):
        """(captures, replays) of the many-cluster call's single graph."""
        c, r = C.c_longlong(), C.c_longlong()
        self.check(self._lib.refeff_fms_context_graph_stats(self.handle, C.byref(c), C.byref(r)))
        return c.value, r.value

    def last_error(self) -> str:
        return self._lib.refeff_fms_last_error(self.handle).decode()

    def check(self, rc: int):
        if rc:
            raise FmsError(rc, self.last_error())

    def close(self):
        if getattr(self, "handle", None):
            self._lib.refeff_fms_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class PlanShape:
    n_states: int
    channel_count: int
    absorber_block: int
    n_potentials: int


class FmsRealSpacePlan:
    """Energy-independent FMS plan resident on the GPU (FmsRealSpacePlan)."""

    def __init__(self, ctx: Context, handle, inputs: dict):
        self.ctx = ctx
        self.handle = handle
        self.inputs = inputs
        n, c, m, npot = (C.c_int() for _ in range(4))
        ctx.check(ctx._lib.refeff_fms_plan_query(handle, C.byref(n), C.byref(c), C.byref(m), C.byref(npot)))
        self.shape = PlanShape(n.value, c.value, m.value, npot.value)

    def set_batch(self, max_batch: int):
        self.ctx.check(self.ctx._lib.refeff_fms_plan_set_batch(self.handle, int(max_batch)))

    def set_tuning(self, inner_width: int = 0, paired_blocks: int = -1):
        """FP32 elimination choices of this plan (refeff_fms_plan_set_tuning)."""
        self.ctx.check(self.ctx._lib.refeff_fms_plan_set_tuning(self.handle, int(inner_width), int(paired_blocks)))

    def tuning(self):
        i, p = C.c_int(), C.c_int()
        self.ctx.check(self.ctx._lib.refeff_fms_plan_get_tuning(self.handle, C.byref(i), C.byref(p)))
        return i.value, p.value

    def set_refinement(self, max_iterations: int, tolerance: float):
        self.ctx.check(self.ctx._lib.refeff_fms_plan_set_refinement(self.handle, int(max_iterations), float(tolerance)))

    def set_profiling(self, enable: bool):
        self.ctx.check(self.ctx._lib.refeff_fms_plan_set_profiling(self.handle, 1 if enable else 0))

    def refinement_stats(self, n_energies: int):
        """(relative residual, corrections, FP64 fallback flag) per energy of the last FP32_REFINED call."""
        rel = np.zeros(n_energies)
        its = np.zeros(n_energies, np.int32)
        fb = np.zeros(n_energies, np.int32)
        self.ctx.check(self.ctx._lib.refeff_fms_plan_refinement_stats(self.handle, int(n_energies), _ptr(rel),
                                                                       _ptr(its), _ptr(fb)))
        return rel, its, fb

    def _points(self, wave_numbers, phase_shifts):
        nsp, L, npot = self.inputs["nsp"], self.inputs["L"], self.inputs["npot"]
        k = np.ascontiguousarray(np.asarray(wave_numbers, dtype=np.complex128).reshape(-1, nsp))
        E = k.shape[0]
        ph = np.asarray(phase_shifts, dtype=np.complex128).reshape(E, nsp, 2 * L + 1, npot)
        xp = np.ascontiguousarray(np.stack([ph[e].reshape(-1, order="F") for e in range(E)])) if E else \
            np.zeros((0,), np.complex128)
        return k, xp, _EnergyPoints(E, _ptr(k), _ptr(xp))

    def set_preconditioner(self, model):
        """Attach a learned preconditioner (PrecondModel) for the BiCGSTAB form, or detach it (None)."""
        self._model = model  # the plan does not own the model: keep it alive here
        self.ctx.check(self.ctx._lib.refeff_fms_plan_set_preconditioner(self.handle,
                                                                         model.handle if model else None))

    def set_precond_window(self, e_lo_ev: float = -1e300, e_hi_ev: float = 1e300):
        """Apply the learned preconditioner only for E - E_ref in [e_lo_ev, e_hi_ev] eV."""
        self.ctx.check(self.ctx._lib.refeff_fms_plan_set_precond_window(self.handle, float(e_lo_ev), float(e_hi_ev)))

    def set_bicgstab(self, max_iterations=400, tolerance=1e-6, poll_interval=8):
        self.ctx.check(self.ctx._lib.refeff_fms_plan_set_bicgstab(self.handle, int(max_iterations),
                                                                   float(tolerance), int(poll_interval)))

    def set_bicgstab_window(self, e_lo_ev: float = -1e300, e_hi_ev: float = 1e300):
        """Iterate the BiCGSTAB form only for E - E_ref in [e_lo_ev, e_hi_ev] eV; other energies go to the refined LU."""
        self.ctx.check(self.ctx._lib.refeff_fms_plan_set_bicgstab_window(self.handle, float(e_lo_ev), float(e_hi_ev)))

    def bicgstab_lu_energies(self, n_energies: int):
        """Per energy of the last BiCGSTAB-form call: 0 BiCGSTAB, 1 missed the tolerance -> refined LU, 2 outside
        the window -> refined LU."""
        fl = np.zeros(n_energies, np.int32)
        self.ctx.check(self.ctx._lib.refeff_fms_plan_bicgstab_lu_energies(self.handle, int(n_energies), _ptr(fl)))
        return fl

    def bicgstab_stats(self, n_energies: int):
        """BiCGSTAB iterations per energy of the last BICGSTAB-form call (initial solve + corrections)."""
        its = np.zeros(n_energies, np.int32)
        self.ctx.check(self.ctx._lib.refeff_fms_plan_bicgstab_stats(self.handle, int(n_energies), _ptr(its)))
        return its

    def precond_features(self, wave_numbers, phase_shifts, model_features: int):
        """Features of every (energy, atom), atoms in device order (absorber last): (E, N, F) float32."""
        k, xp, pts = self._points(wave_numbers, phase_shifts)
        N = len(self.inputs["potentials"])
        out = np.zeros((k.shape[0], N, model_features), np.float32)
        self.ctx.check(self.ctx._lib.refeff_fms_plan_precond_features(self.handle, C.byref(pts), _ptr(out)))
        return out

    def inverse_diagonal(self, wave_numbers, phase_shifts, atom: int):
        """Diagonal of atom `atom`'s block of (I - G0 T)^-1 per energy from the FP64 LU: (E, states) complex."""
        k, xp, pts = self._points(wave_numbers, phase_shifts)
        E = k.shape[0]
        nsp, L = self.inputs["nsp"], self.inputs["L"]
        lm = min(int(self.inputs["lmaxph"][self.inputs["potentials"][atom]]), L)
        lm = L if lm < 0 else lm
        cnt = nsp * (lm + 1) ** 2
        out = np.zeros((E, cnt), np.complex128)
        st = np.zeros(E, np.int32)
        self.ctx.check(self.ctx._lib.refeff_fms_plan_inverse_diagonal(self.handle, C.byref(pts), int(atom), _ptr(out),
                                                                       _ptr(st)))
        return out, st

    def inverse_block(self, wave_numbers, phase_shifts, atom: int):
        """Atom `atom`'s whole block of (I - G0 T)^-1 per energy from the FP64 LU: (E, states, states) complex,
        [e, r, c] = (A^-1)[s0 + r, s0 + c]."""
        k, xp, pts = self._points(wave_numbers, phase_shifts)
        E = k.shape[0]
        nsp, L = self.inputs["nsp"], self.inputs["L"]
        lm = min(int(self.inputs["lmaxph"][self.inputs["potentials"][atom]]), L)
        lm = L if lm < 0 else lm
        cnt = nsp * (lm + 1) ** 2
        out = np.zeros((E, cnt, cnt), np.complex128)
        st = np.zeros(E, np.int32)
        self.ctx.check(self.ctx._lib.refeff_fms_plan_inverse_block(self.handle, C.byref(pts), int(atom), _ptr(out),
                                                                    _ptr(st)))
        return out, st

    PHASES = ("build", "eliminate", "sweeps", "residual", "extract", "tc_update")

    def phase_times(self) -> dict:
        out = np.zeros(len(self.PHASES))
        self.ctx.check(self.ctx._lib.refeff_fms_plan_phase_times(self.handle, _ptr(out), len(out)))
        return dict(zip(self.PHASES, out.tolist()))

    def close(self):
        if getattr(self, "handle", None):
            self.ctx._lib.refeff_fms_real_space_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PRECOND_DIAGONAL = 0
PRECOND_BLOCK = 1


class PrecondModel:
    """The learned preconditioner (refeff_fms_precond_model): an MLP trained and run on the GPU that predicts,
    per (energy, atom), the channel diagonal (kind PRECOND_DIAGONAL) or the whole block (PRECOND_BLOCK) of the
    atom's block of (I - G0 T)^-1 as a deviation from the identity."""

    def __init__(self, ctx: Context, lmax: int, hidden: int = 64, seed: int = 0, kind: int = PRECOND_DIAGONAL):
        self.ctx = ctx
        h = _p()
        ctx.check(ctx._lib.refeff_fms_precond_model_create_kind(ctx.handle, int(lmax), int(hidden), int(kind),
                                                                C.c_ulonglong(seed), C.byref(h)))
        self.handle = h
        self.lmax = int(lmax)
        self.kind = int(kind)
        f, hd, o, npar = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        ctx.check(ctx._lib.refeff_fms_precond_model_query(h, C.byref(f), C.byref(hd), C.byref(o), C.byref(npar)))
        self.n_features, self.hidden, self.n_outputs, self.n_params = f.value, hd.value, o.value, npar.value

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        self.ctx.check(self.ctx._lib.refeff_fms_precond_get_params(self.handle, _ptr(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        self.ctx.check(self.ctx._lib.refeff_fms_precond_set_params(self.handle, _ptr(p)))

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        loss = C.c_double()
        g = np.zeros(self.n_params, np.float32)
        self.ctx.check(self.ctx._lib.refeff_fms_precond_loss_grad(self.handle, X.shape[0], _ptr(X), _ptr(T),
                                                                  C.byref(loss), _ptr(g)))
        return loss.value, g

    def train(self, X, T, *, epochs=200, batch_size=256, learning_rate=2e-3, seed=0):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        hist = np.zeros(max(epochs, 1))
        self.ctx.check(self.ctx._lib.refeff_fms_precond_train(self.handle, X.shape[0], _ptr(X), _ptr(T), int(epochs),
                                                              int(batch_size), C.c_float(learning_rate),
                                                              C.c_ulonglong(seed), _ptr(hist)))
        return hist[:epochs]

    def predict(self, X):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((X.shape[0], self.n_outputs), np.float32)
        self.ctx.check(self.ctx._lib.refeff_fms_precond_predict(self.handle, X.shape[0], _ptr(X), _ptr(Y)))
        return Y

    def close(self):
        if getattr(self, "handle", None):
            self.ctx._lib.refeff_fms_precond_model_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fms_real_space_plan(ctx: Context, positions, potentials, raw_potential_lmax, *, spin_channels=1, spin_selector=0,
                        lfms=0, minv=0, global_lmax=None, direct_cutoff=1.0e6, mean_square_displacements=None,
                        sig2g=0.0, convergence_tolerance=1.0e-3, zero_tolerance=0.0,
                        full_scattering=False) -> FmsRealSpacePlan:
    """Energy-independent plan (fms_real_space_plan, crates/refeff-core/src/fms/driver.rs:105-140).

    full_scattering: request the full matrix (I - G0 T)^-1 G0 (fms.inp save_gg_slice), which forces the LU form;
    solve such a plan with fms_full_scattering_spectrum.
    """
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
    pots = np.ascontiguousarray(potentials, dtype=np.int32)
    lmax = np.ascontiguousarray(raw_potential_lmax, dtype=np.int32)
    L = int(lmax.max()) if global_lmax is None else int(global_lmax)
    msd = None if mean_square_displacements is None else np.asfortranarray(mean_square_displacements, dtype=np.float32)
    inp = _PlanInput(len(pots), _ptr(pos), _ptr(pots), int(spin_channels), int(spin_selector), int(lfms), int(minv),
                     len(lmax) - 1, L, _ptr(lmax), float(direct_cutoff), _ptr(msd), float(sig2g),
                     float(convergence_tolerance), float(zero_tolerance))
    h = _p()
    create = ctx._lib.refeff_fms_real_space_plan_create_full if full_scattering else \
        ctx._lib.refeff_fms_real_space_plan_create
    ctx.check(create(ctx.handle, C.byref(inp), C.byref(h)))
    return FmsRealSpacePlan(ctx, h, dict(positions=pos, potentials=pots, lmaxph=lmax, nsp=int(spin_channels),
                                          L=L, npot=len(lmax)))


def _energy_inputs(plan: FmsRealSpacePlan, wave_numbers, phase_shifts):
    nsp, L, npot = plan.inputs["nsp"], plan.inputs["L"], plan.inputs["npot"]
    k = np.ascontiguousarray(np.asarray(wave_numbers, dtype=np.complex128).reshape(-1, nsp))
    E = k.shape[0]
    ph = np.asarray(phase_shifts, dtype=np.complex128).reshape(E, nsp, 2 * L + 1, npot)
    xp = np.ascontiguousarray(np.stack([ph[e].reshape(-1, order="F") for e in range(E)])) if E else \
        np.zeros((0,), np.complex128)
    return k, xp, E


def fms_full_scattering_spectrum(plan: FmsRealSpacePlan, wave_numbers, phase_shifts):
    """Spectrum of a full-scattering plan with the FP64 LU: (tables (E, C, C, npot), slice (E, b, n),
    diag (E, N, b, b), status (E,)), b = nsp (L+1)^2; slice and diag are the save_gg_slice outputs of
    build_saved_fms_scattering_outputs (crates/refeff-engine/src/fms.rs:4154-4216), reference state order."""
    npot = plan.inputs["npot"]
    k, xp, E = _energy_inputs(plan, wave_numbers, phase_shifts)
    Cc, n, N = plan.shape.channel_count, plan.shape.n_states, len(plan.inputs["potentials"])
    out = np.zeros(E * Cc * Cc * npot, dtype=np.complex128)
    sl = np.zeros(E * Cc * n, dtype=np.complex128)
    dg = np.zeros(E * N * Cc * Cc, dtype=np.complex128)
    status = np.zeros(E, dtype=np.int32)
    pts = _EnergyPoints(E, _ptr(k), _ptr(xp))
    rc = plan.ctx._lib.refeff_fms_real_space_spectrum_full(plan.handle, C.byref(pts), _ptr(out), _ptr(sl), _ptr(dg),
                                                           _ptr(status), None)
    if rc:
        raise FmsError(rc, plan.ctx.last_error())
    tabs = out.reshape(E, Cc * Cc * npot)
    scat = np.stack([tabs[e].reshape((Cc, Cc, npot), order="F") for e in range(E)]) if E else \
        np.zeros((0, Cc, Cc, npot), np.complex128)
    slice_ = sl.reshape(E, n, Cc).transpose(0, 2, 1)
    diag = dg.reshape(E, N, Cc, Cc).transpose(0, 1, 3, 2)
    return scat, slice_, diag, status


def fms_real_space_spectrum(plan: FmsRealSpacePlan, wave_numbers, phase_shifts, form=FORM_FP64_LU,
                            raise_on_error=True):
    """Scattering tables (E, C, C, npot) complex128 and per-energy status codes.

    wave_numbers: (E, nsp) complex; phase_shifts: (E, nsp, 2L+1, npot) complex (FEFF xphase per energy).
    """
    nsp, L, npot = plan.inputs["nsp"], plan.inputs["L"], plan.inputs["npot"]
    k = np.ascontiguousarray(np.asarray(wave_numbers, dtype=np.complex128).reshape(-1, nsp))
    E = k.shape[0]
    ph = np.asarray(phase_shifts, dtype=np.complex128).reshape(E, nsp, 2 * L + 1, npot)
    xp = np.ascontiguousarray(np.stack([ph[e].reshape(-1, order="F") for e in range(E)])) if E else \
        np.zeros((0,), np.complex128)
    Cc = plan.shape.channel_count
    out = np.zeros(E * Cc * Cc * npot, dtype=np.complex128)
    status = np.zeros(E, dtype=np.int32)
    pts = _EnergyPoints(E, _ptr(k), _ptr(xp))
    rep = _Report()
    rc = plan.ctx._lib.refeff_fms_real_space_spectrum(plan.handle, C.byref(pts), int(form), _ptr(out), _ptr(status),
                                                      C.byref(rep))
    if rc and (raise_on_error or rc not in (9, 10, 6, 8, 19)):
        raise FmsError(rc, plan.ctx.last_error())
    tabs = out.reshape(E, Cc * Cc * npot)
    scat = np.stack([tabs[e].reshape((Cc, Cc, npot), order="F") for e in range(E)]) if E else \
        np.zeros((0, Cc, Cc, npot), np.complex128)
    return scat, status


def fms_real_space_spectrum_device(plan: FmsRealSpacePlan, d_k: int, d_phase: int, n_energies: int, d_gg: int,
                                   d_status: int, form=FORM_FP64_LU, stream: int = 0):
    """Device-pointer variant (pointers as ints, e.g. torch tensor .data_ptr())."""
    rc = plan.ctx._lib.refeff_fms_real_space_spectrum_device(plan.handle, int(n_energies), _p(d_k), _p(d_phase),
                                                             int(form), _p(d_gg), _p(d_status),
                                                             _p(stream) if stream else None)
    if rc:
        raise FmsError(rc, plan.ctx.last_error())


def gg_section(plan: FmsRealSpacePlan, scattering_table, nspu: int | None = None):
    nsp = plan.inputs["nsp"]
    nspu = nsp if nspu is None else int(nspu)
    tab = np.asfortranarray(scattering_table, dtype=np.complex128)
    lmax0 = int(round((plan.shape.absorber_block // nsp) ** 0.5)) - 1
    w = nspu * (lmax0 + 1) ** 2
    out = np.zeros(w * w, dtype=np.complex128)
    flat = np.ascontiguousarray(tab.reshape(-1, order="F"))
    rc = plan.ctx._lib.refeff_fms_gg_section(plan.handle, _ptr(flat), nspu, _ptr(out))
    if rc:
        raise FmsError(rc)
    return out.reshape((w, w), order="F")


def complex_lu_solve_batched(ctx: Context, A, B, form=FORM_FP64_LU):
    """Solve A[b] X[b] = B[b] for a batch (batch, n, n) / (batch, n, m) complex; returns X, status, pivot."""
    A = np.asarray(A, dtype=np.complex128)
    B = np.asarray(B, dtype=np.complex128)
    if A.ndim == 2:
        A = A[None]
    if B.ndim == 2:
        B = B[None]
    batch, n, _ = A.shape
    m = B.shape[2]
    a = np.ascontiguousarray(np.stack([A[i].reshape(-1, order="F") for i in range(batch)]))
    b = np.ascontiguousarray(np.stack([B[i].reshape(-1, order="F") for i in range(batch)]))
    x = np.zeros_like(b)
    st = np.zeros(batch, np.int32)
    piv = np.zeros(batch, np.int32)
    rc = ctx._lib.refeff_complex_lu_solve_batched(ctx.handle, n, m, batch, _ptr(a), _ptr(b), _ptr(x), int(form),
                                                  _ptr(st), _ptr(piv))
    X = np.stack([x[i].reshape((n, m), order="F") for i in range(batch)])
    if rc and rc not in (9, 10):
        raise FmsError(rc, ctx.last_error())
    return X, st, piv


def run_fms_in_dir(ctx: Context, work_dir, form=FORM_FP64_LU) -> dict:
    """The `fms` stage on a FEFF work directory (run_fms_in_dir, crates/refeff-engine/src/fms.rs:1102-1127):
    reads fms.inp, global.inp, phase.bin, geom.dat (and .dimensions.dat if present) and writes gg.bin, gg.dat
    and log3.dat.  Returns the run report as a dict."""
    rep = _Report()
    rc = ctx._lib.refeff_fms_run_dir(ctx.handle, str(work_dir).encode(), int(form), C.byref(rep))
    if rc:
        raise FmsError(rc, ctx.last_error())
    return {"seconds": rep.seconds, "refinement_iterations": rep.refinement_iterations,
            "residual_max": rep.residual_max, "energies_failed": rep.energies_failed,
            "fp64_fallbacks": rep.fp64_fallbacks}


def write_gg_dat(path, sections) -> None:
    """Write square complex sections (n, dim, dim) as FEFF gg.dat text (crates/refeff-io/src/gg_dat.rs:174-202)."""
    lib = load()
    sec = np.asarray(sections, dtype=np.complex128)
    n, dim, _ = sec.shape
    flat = np.ascontiguousarray(np.stack([sec[i].reshape(-1, order="F") for i in range(n)])) if n else \
        np.zeros(0, np.complex128)
    rc = lib.refeff_fms_write_gg_dat(str(path).encode(), n, dim, _ptr(flat))
    if rc:
        raise FmsError(rc, f"cannot write {path}")


def ff2x_xanes_mu(*, energy, ne1, fermi_index, omega, cross_section, background, trace, s02=1.0, ispec=1,
                  absolu=0, include_atomic=True, real_correction=0.0, imaginary_correction=0.0,
                  fermi_photon_energy=0.0, electronic_temperature=0.0):
    """FF2X XANES mu(E) from the MKGTR trace (crates/refeff-engine/src/ff2x.rs:3186-3262, 3309-3399, 4437-5050):
    returns (mu, mu0, chi) over the ne1 main rows.  energy, cross_section, trace: ne complex; background: ne
    reals; omega: ne1 photon energies; all energies in Hartree; electronic_temperature in eV (> 0: the thermal
    xscorr).  Host only."""
    lib = load()
    e = np.ascontiguousarray(energy, dtype=np.complex128)
    ne = e.shape[0]
    om = np.ascontiguousarray(omega, dtype=np.float64)
    xs = np.ascontiguousarray(cross_section, dtype=np.complex128)
    bg = np.ascontiguousarray(background, dtype=np.float64)
    tr = np.ascontiguousarray(trace, dtype=np.complex128)
    if om.shape[0] < ne1 or xs.shape[0] != ne or bg.shape[0] != ne or tr.shape[0] != ne:
        raise FmsError(1, "ff2x_xanes_mu: array lengths do not match ne / ne1")
    mu, mu0, chi = (np.zeros(int(ne1)) for _ in range(3))
    rc = lib.refeff_ff2x_xanes_mu_thermal(ne, int(ne1), int(fermi_index), int(ispec), int(absolu),
                                          int(bool(include_atomic)), _ptr(e), _ptr(om), _ptr(xs), _ptr(bg), _ptr(tr),
                                          float(s02), float(real_correction), float(imaginary_correction),
                                          float(fermi_photon_energy), float(electronic_temperature), _ptr(mu),
                                          _ptr(mu0), _ptr(chi))
    if rc:
        raise FmsError(rc, "ff2x_xanes_mu")
    return mu, mu0, chi


def ff2x_xscorr(*, energy, ne1, fermi_index, cross_section, background, path_chi, ispec=1, real_correction=0.0,
                electronic_temperature=0.0):
    """FF2X xscorr (crates/refeff-engine/src/ff2x.rs:4437-5050): the correction cchi (ne1 complex) of
    xmu = cross_section + path_chi * background over the xsect.dat rows; the thermal form when
    electronic_temperature (eV) > 0.  Host only."""
    lib = load()
    e = np.ascontiguousarray(energy, dtype=np.complex128)
    ne = e.shape[0]
    xs = np.ascontiguousarray(cross_section, dtype=np.complex128)
    bg = np.ascontiguousarray(background, dtype=np.float64)
    pc = np.ascontiguousarray(path_chi, dtype=np.complex128)
    if xs.shape[0] != ne or bg.shape[0] != ne or pc.shape[0] != ne:
        raise FmsError(1, "ff2x_xscorr: array lengths do not match the energy rows")
    out = np.zeros(int(ne1), np.complex128)
    rc = lib.refeff_ff2x_xscorr(ne, int(ne1), int(fermi_index), int(ispec), _ptr(e), _ptr(xs), _ptr(bg), _ptr(pc),
                                float(real_correction), float(electronic_temperature), _ptr(out))
    if rc:
        raise FmsError(rc, "ff2x_xscorr")
    return out


def reciprocal_integrate(ctx: Context, structure_factors, weights, t_matrix, form=FORM_FP64_LU,
                         raise_on_error=True):
    """Reciprocal-space FMS of one energy (crates/refeff-core/src/fms/reciprocal.rs:67-223): the weighted
    k-point average of (I - G(k) T)^-1 G(k) on the GPU.  structure_factors: (K, n, n) complex; weights: (K,);
    t_matrix: (n, n).  Returns (green (n, n), per-k-point status)."""
    G = np.asarray(structure_factors, dtype=np.complex128)
    K, n, _ = G.shape
    g = np.ascontiguousarray(G.transpose(0, 2, 1))  # column-major per k-point
    w = np.ascontiguousarray(weights, dtype=np.float64)
    t = np.asfortranarray(t_matrix, dtype=np.complex128)
    out = np.zeros((n, n), dtype=np.complex128, order="F")
    st = np.zeros(K, np.int32)
    rc = ctx._lib.refeff_fms_reciprocal_integrate(ctx.handle, n, K, _ptr(g), _ptr(w), _ptr(t), int(form), _ptr(out),
                                                  _ptr(st))
    if rc and raise_on_error:
        raise FmsError(rc, ctx.last_error())
    return np.array(out), st


def reciprocal_core_hole(green, absorber_offset, t_difference):
    """FEFF kkrintegral core-hole Dyson update (reciprocal.rs:236-302), host FP64."""
    lib = load()
    G = np.asfortranarray(green, dtype=np.complex128)
    C = np.asfortranarray(t_difference, dtype=np.complex128)
    n, b = G.shape[0], C.shape[0]
    out = np.zeros((n, n), dtype=np.complex128, order="F")
    rc = lib.refeff_fms_reciprocal_core_hole(n, _ptr(G), int(absorber_offset), b, _ptr(C), _ptr(out))
    if rc:
        raise FmsError(rc, "reciprocal core hole")
    return np.array(out)


def ff2x_debye_factor(wave_number, sig_gk, mu0, chi):
    """FF2X's sig_gk Debye factor on chi (refeff_ff2x_debye_factor): returns (mu, chi)."""
    k = np.ascontiguousarray(wave_number, np.float64)
    c = np.array(chi, np.float64)
    m0 = np.ascontiguousarray(mu0, np.float64)
    mu = np.zeros_like(c)
    rc = load().refeff_ff2x_debye_factor(len(k), _ptr(k), float(sig_gk), _ptr(m0), _ptr(c), _ptr(mu))
    if rc:
        raise FmsError(rc, "ff2x debye factor")
    return mu, c


def ff2x_lorentz_convolve(omega, spectrum, width):
    """FEFF conv (crates/refeff-core/src/convolution/lorentzian.rs:32-100), host only."""
    lib = load()
    om = np.ascontiguousarray(omega, dtype=np.float64)
    y = np.ascontiguousarray(spectrum, dtype=np.complex128)
    out = np.zeros_like(y)
    rc = lib.refeff_ff2x_lorentz_convolve(int(om.shape[0]), _ptr(om), _ptr(y), float(width), _ptr(out))
    if rc:
        raise FmsError(rc, "ff2x_lorentz_convolve")
    return out


def write_gg_slice_bin(path, values) -> None:
    """FEFF gg_slice.bin from (ne, rows, cols) complex values (crates/refeff-io/src/rhorrp_gg_bin.rs:138-160)."""
    lib = load()
    v = np.asarray(values, dtype=np.complex128)
    ne, rows, cols = v.shape
    flat = np.ascontiguousarray(v.transpose(0, 2, 1))
    rc = lib.refeff_fms_write_gg_slice_bin(str(path).encode(), ne, rows, cols, _ptr(flat))
    if rc:
        raise FmsError(rc, f"cannot write {path}")


def write_gg_diag_bin(path, values) -> None:
    """FEFF gg_diag.bin from (ne, atoms, dim, dim) complex values (crates/refeff-io/src/rhorrp_gg_bin.rs:228-252)."""
    lib = load()
    v = np.asarray(values, dtype=np.complex128)
    ne, na, dim, _ = v.shape
    flat = np.ascontiguousarray(v.transpose(0, 1, 3, 2))
    rc = lib.refeff_fms_write_gg_diag_bin(str(path).encode(), ne, na, dim, _ptr(flat))
    if rc:
        raise FmsError(rc, f"cannot write {path}")


def geometry_from_feff_inp(path):
    """The cluster of a feff.inp as FEFF's rdinp hands it to the FMS stage (refeff_fms_geometry_from_feff_inp):
    returns (xyz (n, 3) float64, ipot (n,) int32, model_atoms (nph + 1,) int32); row 0 is the absorber."""
    lib = load()
    n, nm = C.c_int32(), C.c_int32()
    b = str(path).encode()
    rc = lib.refeff_fms_geometry_from_feff_inp(b, 0, None, None, C.byref(n), 0, None, C.byref(nm))
    if rc:
        raise FmsError(rc, lib.refeff_fms_feff_inp_last_error().decode())
    xyz = np.zeros((n.value, 3))
    ipot = np.zeros(n.value, np.int32)
    model = np.zeros(nm.value, np.int32)
    rc = lib.refeff_fms_geometry_from_feff_inp(b, n.value, _ptr(xyz), _ptr(ipot), C.byref(n), nm.value, _ptr(model),
                                               C.byref(nm))
    if rc:
        raise FmsError(rc, lib.refeff_fms_feff_inp_last_error().decode())
    return xyz, ipot, model


def ff2x_read_xsect_dat(path, s02=1.0, mbconv=0) -> dict:
    """XSPH's xsect.dat handed to FF2X as FEFF's rdxbin does (refeff_ff2x_read_xsect_dat): energies in Hartree,
    omega, signed wave numbers, background (xsnorm), cross section, ne1, the zero-based Fermi index and the
    effective S02 (the file's when mbconv > 0 or s02 <= 0.1)."""
    lib = load()
    b = str(path).encode()
    counts = np.zeros(4, np.int32)
    rc = lib.refeff_ff2x_read_xsect_dat(b, float(s02), int(mbconv), 0, _ptr(counts), None, None, None, None, None,
                                        None)
    if rc:
        raise FmsError(rc, lib.refeff_ff2x_xsect_last_error().decode())
    n = int(counts[0])
    sc = np.zeros(7)
    energy = np.zeros(n, np.complex128)
    omega, wave, background = np.zeros(n), np.zeros(n), np.zeros(n)
    xsec = np.zeros(n, np.complex128)
    rc = lib.refeff_ff2x_read_xsect_dat(b, float(s02), int(mbconv), n, _ptr(counts), _ptr(sc), _ptr(energy),
                                        _ptr(omega), _ptr(wave), _ptr(background), _ptr(xsec))
    if rc:
        raise FmsError(rc, lib.refeff_ff2x_xsect_last_error().decode())
    return {"rows": n, "ne1": int(counts[1]), "fermi_index": int(counts[2]), "titles": int(counts[3]),
            "s02": sc[0], "file_s02": sc[1], "erelax": sc[2], "wp": sc[3], "edge": sc[4], "emu": sc[5],
            "core_hole_width": sc[6], "energy": energy, "omega": omega, "wave_number": wave,
            "background": background, "cross_section": xsec}


def write_geom_dat(feff_inp, geom_dat) -> None:
    """geom.dat for the cluster of a feff.inp, byte-compatible with FEFF rdinp's writer."""
    lib = load()
    rc = lib.refeff_fms_write_geom_dat(str(feff_inp).encode(), str(geom_dat).encode())
    if rc:
        raise FmsError(rc, lib.refeff_fms_feff_inp_last_error().decode())


def read_phase_bin(path) -> dict:
    """Decode a FEFF phase.bin (crates/refeff-io/src/phase_bin/parse.rs:18-130).

    Returns energy_grid (ne,), reference_energy (ne, nsp), potential_lmax (npot,) and phase_shifts
    (ne, 2*lmax_max+1, nsp, npot) with the signed-l axis centred on lmax_max."""
    lib = load()
    nsp, ne, npot, lm = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    rc = lib.refeff_fms_phase_bin_dims(str(path).encode(), C.byref(nsp), C.byref(ne), C.byref(npot), C.byref(lm))
    if rc:
        raise FmsError(rc, f"cannot read {path}")
    nsp, ne, npot, lm = nsp.value, ne.value, npot.value, lm.value
    grid = np.zeros(ne, np.complex128)
    eref = np.zeros(ne * nsp, np.complex128)
    lmax = np.zeros(npot, np.int32)
    ph = np.zeros(ne * (2 * lm + 1) * nsp * npot, np.complex128)
    rc = lib.refeff_fms_phase_bin_read(str(path).encode(), _ptr(grid), _ptr(eref), _ptr(lmax), _ptr(ph))
    if rc:
        raise FmsError(rc, f"cannot read {path}")
    return {"energy_grid": grid, "reference_energy": eref.reshape((ne, nsp), order="F"), "potential_lmax": lmax,
            "phase_shifts": ph.reshape((ne, 2 * lm + 1, nsp, npot), order="F")}


NOALLOC_SCRATCH_BYTES = 24 * 1024 * 1024


def complex_lu_solve_device_noalloc(n: int, m: int, batch: int, d_A: int, d_B: int, d_X: int, d_status: int = 0,
                                    d_pivot: int = 0, stream: int = 0) -> None:
    """Allocation-free FP64 batched solve on device pointers (ints, e.g. torch ``.data_ptr()``), asynchronous on
    ``stream``; scratch is the library's static device array (NOALLOC_SCRATCH_BYTES).  No reference counterpart."""
    lib = load()
    fn = lib.refeff_complex_lu_solve_device_noalloc
    fn.argtypes = [_i, _i, _i, _p, _p, _p, _p, _p, _p]
    fn.restype = _i
    rc = fn(int(n), int(m), int(batch), _p(d_A), _p(d_B), _p(d_X), _p(d_status) if d_status else None,
            _p(d_pivot) if d_pivot else None, _p(stream) if stream else None)
    if rc:
        raise FmsError(rc, "allocation-free dense solve")


def debye_sigma2_table(ctx: Context, idwopt, positions, potentials, atomic_numbers, *, temperature,
                       debye_temperature, average_norman_radius, sig2g=0.0, with_debye_term=False):
    """Pair sigma^2 table of the FMS stage on the GPU (refeff_fms_debye_sigma2_table; the reference's
    fms_mean_square_displacements_with_metadata, crates/refeff-engine/src/fms.rs:4345-4433, for idwopt < 0, 0 and
    3).  Returns the f32 (N, N) table indexed [atom2, atom1] (and the FP64 Debye term when asked)."""
    lib = load()
    pos = np.ascontiguousarray(np.asarray(positions, np.float32).reshape(-1, 3))
    pots = np.ascontiguousarray(np.asarray(potentials, np.int32))
    z = np.ascontiguousarray(np.asarray(atomic_numbers, np.int32))
    N = pos.shape[0]
    out = np.zeros(N * N, np.float32)
    term = np.zeros(N * N) if with_debye_term else None
    rc = lib.refeff_fms_debye_sigma2_table(ctx.handle, int(idwopt), N, _ptr(pos), _ptr(pots), len(z), _ptr(z),
                                           float(temperature), float(debye_temperature),
                                           float(average_norman_radius), C.c_float(sig2g), _ptr(out), _ptr(term))
    if rc:
        raise FmsError(rc, ctx.last_error())
    table = out.reshape((N, N), order="F")
    return (table, term.reshape((N, N), order="F")) if with_debye_term else table


def transition_matrix(*, lmax, initial_kappa, polarization, polarization_tensor=None, multipole=1,
                      trace_orbital=False, spin=1, spin_channels=1, spin_vector_angle=0.0):
    """FEFF bcoef (transition_b_matrix, crates/refeff-core/src/angular/transition.rs:9-73).

    Returns (bmat, lind, kiind); bmat has shape (2L+1, 2, 8, 2L+1, 2, 8) indexed [m2+L, s2, k2, m1+L, s1, k1]."""
    lib = load()
    ML = 2 * lmax + 1
    out = np.zeros(ML * 2 * 8 * ML * 2 * 8, np.complex128)
    ptz = None if polarization_tensor is None else np.ascontiguousarray(
        np.asarray(polarization_tensor, np.complex128).reshape(3, 3))
    lind = np.zeros(8, np.int32)
    kiind = np.zeros(8, np.int32)
    rc = lib.refeff_fms_transition_matrix(int(lmax), int(initial_kappa), int(polarization), _ptr(ptz), int(multipole),
                                          int(bool(trace_orbital)), int(spin), int(spin_channels),
                                          float(spin_vector_angle), _ptr(out), _ptr(lind), _ptr(kiind))
    if rc:
        raise FmsError(rc, "transition matrix")
    return out.reshape((ML, 2, 8, ML, 2, 8), order="F"), lind, kiind


def mkgtr_trace(ctx: Context, gg, bmats, linds, rkk, *, active_spin_channels, lmax):
    """getgtr trace on the GPU (crates/refeff-core/src/fms/mkgtr.rs:790-952).

    gg (E, dim, dim), bmats / linds one per spectrum, rkk (E, 8, nsp) -> traces (n_spectra, E)."""
    gg = np.asarray(gg, np.complex128)
    E, dim, _ = gg.shape
    g = np.ascontiguousarray(np.stack([gg[e].reshape(-1, order="F") for e in range(E)]))
    b = np.ascontiguousarray(np.concatenate([np.asarray(x, np.complex128).reshape(-1, order="F") for x in bmats]))
    li = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int32) for x in linds]))
    rk = np.asarray(rkk, np.complex128)
    r = np.ascontiguousarray(rk.reshape(-1, order="F"))
    nspec = len(bmats)
    out = np.zeros(nspec * E, np.complex128)
    rc = ctx._lib.refeff_fms_mkgtr_trace(ctx.handle, E, dim, int(active_spin_channels), int(lmax), nspec, _ptr(li),
                                         _ptr(b), _ptr(g), _ptr(r), int(rk.shape[2]), _ptr(out))
    if rc:
        raise FmsError(rc, ctx.last_error())
    return out.reshape((nspec, E), order="F")


def mkgtr_trace_device(ctx: Context, n_energies, dim, active_spin_channels, lmax, bmats, linds, d_gg: int, gg_ld,
                       gg_energy_stride, d_rkk: int, d_traces: int, stream: int = 0):
    """Device-pointer trace (pointers as ints), reading gg[e](r, c) = d_gg[e*stride + r + ld*c]."""
    b = np.ascontiguousarray(np.concatenate([np.asarray(x, np.complex128).reshape(-1, order="F") for x in bmats]))
    li = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int32) for x in linds]))
    rc = ctx._lib.refeff_fms_mkgtr_trace_device(ctx.handle, int(n_energies), int(dim), int(active_spin_channels),
                                                int(lmax), len(bmats), _ptr(li), _ptr(b), _p(d_gg), int(gg_ld),
                                                int(gg_energy_stride), _p(d_rkk), _p(d_traces),
                                                _p(stream) if stream else None)
    if rc:
        raise FmsError(rc, ctx.last_error())


def run_mkgtr_in_dir(ctx: Context, work_dir) -> int:
    """The `mkgtr` stage on a FEFF work directory (run_mkgtr_in_dir, crates/refeff-engine/src/fms.rs:559-632):
    gg.bin + phase.bin + global.inp -> fms.bin, gtr.dat, log3.dat.  Returns the number of trace files written."""
    n = C.c_int()
    rc = ctx._lib.refeff_fms_run_mkgtr_dir(ctx.handle, str(work_dir).encode(), C.byref(n))
    if rc:
        raise FmsError(rc, ctx.last_error())
    return n.value


def write_fms_bin(path, traces, *, cluster_radius, ne1=None, ne3=0, nph, pad_width=8) -> None:
    """FEFF fms.bin text (crates/refeff-io/src/fms_bin.rs:77-98); traces (n_spectra, ne)."""
    lib = load()
    tr = np.asarray(traces, np.complex128)
    nspec, ne = tr.shape
    flat = np.ascontiguousarray(tr.reshape(-1, order="F"))
    rc = lib.refeff_fms_write_fms_bin(str(path).encode(), float(cluster_radius), ne, ne if ne1 is None else int(ne1),
                                      int(ne3), int(nph), int(pad_width), nspec, _ptr(flat))
    if rc:
        raise FmsError(rc, f"cannot write {path}")


def write_gtr_dat(path, energy, trace) -> None:
    """FEFF gtr.dat text (crates/refeff-io/src/gtr_dat.rs:60-71)."""
    lib = load()
    e = np.ascontiguousarray(energy, np.complex128)
    t = np.ascontiguousarray(trace, np.complex128)
    rc = lib.refeff_fms_write_gtr_dat(str(path).encode(), len(e), _ptr(e), _ptr(t))
    if rc:
        raise FmsError(rc, f"cannot write {path}")


def fms_real_space_spectrum_multi(plans, wave_numbers, phase_shifts, form=FORM_FP64_LU, raise_on_error=True):
    """Many clusters in one call (refeff_fms_real_space_spectrum_multi): plans[i] with wave_numbers[i]
    (E_i, nsp) and phase_shifts[i] (E_i, nsp, 2L+1, npot); returns lists of scattering tables and statuses."""
    if not plans:
        return [], []
    ctx = plans[0].ctx
    keep, outs, sts = [], [], []
    pts = (_EnergyPoints * len(plans))()
    for i, plan in enumerate(plans):
        nsp, L, npot = plan.inputs["nsp"], plan.inputs["L"], plan.inputs["npot"]
        k = np.ascontiguousarray(np.asarray(wave_numbers[i], dtype=np.complex128).reshape(-1, nsp))
        E = k.shape[0]
        ph = np.asarray(phase_shifts[i], dtype=np.complex128).reshape(E, nsp, 2 * L + 1, npot)
        xp = np.ascontiguousarray(np.stack([ph[e].reshape(-1, order="F") for e in range(E)])) if E else \
            np.zeros((0,), np.complex128)
        Cc = plan.shape.channel_count
        outs.append(np.zeros(E * Cc * Cc * npot, dtype=np.complex128))
        sts.append(np.zeros(E, dtype=np.int32))
        keep += [k, xp]
        pts[i] = _EnergyPoints(E, _ptr(k), _ptr(xp))
    hs = (_p * len(plans))(*[p.handle for p in plans])
    op = (_p * len(plans))(*[_ptr(o) for o in outs])
    sp = (_p * len(plans))(*[_ptr(x) for x in sts])
    rep = _Report()
    rc = ctx._lib.refeff_fms_real_space_spectrum_multi(ctx.handle, len(plans), hs, pts, int(form), op, sp, C.byref(rep))
    if rc and (raise_on_error or rc not in (9, 10, 6, 8, 19)):
        raise FmsError(rc, ctx.last_error())
    tables = []
    for plan, o, x in zip(plans, outs, sts):
        Cc, npot, E = plan.shape.channel_count, plan.inputs["npot"], len(x)
        t = o.reshape(E, Cc * Cc * npot)
        tables.append(np.stack([t[e].reshape((Cc, Cc, npot), order="F") for e in range(E)]) if E else
                      np.zeros((0, Cc, Cc, npot), np.complex128))
    return tables, sts


def autotune_multi(plans, wave_numbers, phase_shifts, form=FORM_FP32_REFINED, sample_energies=16, cache_path=None):
    """Tune the many-cluster call for these plans (refeff_fms_autotune_multi): per size bucket the inner panel
    width and block pairing, then the stream count; cached under cache_path.  Returns a dict of the choice."""
    ctx = plans[0].ctx
    keep, pts = [], (_EnergyPoints * len(plans))()
    for i, plan in enumerate(plans):
        nsp, L, npot = plan.inputs["nsp"], plan.inputs["L"], plan.inputs["npot"]
        k = np.ascontiguousarray(np.asarray(wave_numbers[i], dtype=np.complex128).reshape(-1, nsp))
        E = k.shape[0]
        ph = np.asarray(phase_shifts[i], dtype=np.complex128).reshape(E, nsp, 2 * L + 1, npot)
        x = np.ascontiguousarray(np.stack([ph[e].reshape(-1, order="F") for e in range(E)])) if E else \
            np.zeros((0, nsp * (2 * L + 1) * npot), np.complex128)
        keep += [k, x]
        pts[i].n_energies, pts[i].wave_numbers, pts[i].phase_shifts = E, _ptr(k), _ptr(x)
    handles = (_p * len(plans))(*[p.handle for p in plans])
    out = _Tuning()
    path = None if cache_path is None else str(cache_path).encode()
    ctx.check(ctx._lib.refeff_fms_autotune_multi(ctx.handle, len(plans), handles, pts, int(form), int(sample_energies),
                                                 path, C.byref(out)))
    return {"streams": out.streams, "buckets": out.buckets, "seconds_default": out.seconds_default,
            "seconds_tuned": out.seconds_tuned, "from_cache": bool(out.from_cache)}
