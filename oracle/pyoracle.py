"""TEST INFRASTRUCTURE ONLY: ctypes loader for the CPU oracle (oracle/fms_oracle.cpp).

The oracle restates refeff's real-space FMS arithmetic on the CPU.  Only the
tests, the smoke check and bench.py's CPU-baseline leg may load it; the product
library never does.  ``mode=0`` is the f32-faithful restatement of the
reference's Complex32 path, ``mode=1`` the FP64 oracle.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "build" / "liboracle_fms.so"

F32, F64 = 0, 1

_lib = None


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (g++, OpenMP, -ffp-contract=off)."""
    newest = max((HERE / f).stat().st_mtime for f in ("fms_oracle.cpp", "mkgtr_oracle.cpp", "debye_oracle.cpp", "Makefile"))
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < newest:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


_p = C.c_void_p
_i = C.c_int
_d = C.c_double


def _declare(L):
    sig = {
        "oracle_sort_atoms_by_radius": [_i, _p, _p, _p],
        "oracle_yprep_cluster": [_i, _i, _p, _p, C.c_float, _i, _p, _p, _p, _p, _p],
        "oracle_sort_representative_atoms": [_i, _i, _i, _p, _p, _p],
        "oracle_pair_polar_angles": [_i, _p, _p, _i, _p, _p],
        "oracle_rotation_matrix": [_i, _i, _i, _d, _d, _i, _p],
        "oracle_polynomials": [_i, _i, _i, _i, _p, _p],
        "oracle_t_matrix_phase": [_i, _p, _p],
        "oracle_prefactor": [_i, _p, _p, _d, _p],
        "oracle_lu_factor_solve": [_i, _i, _p, _i, _p, _p, _p],
        "oracle_fms_spectrum": [_i, _i, _p, _p, _i, _i, _i, _i, _i, _p, _d, _p, _d, _i, _p, _p, _p, _p, _i],
        "oracle_driver_setup": [_i, _p, _i, _i, _i, _i, _p, _p, _p, _p, _p, _p, _i],
        "oracle_fms_energy_intermediates": [_i, _i, _p, _p, _i, _i, _i, _i, _i, _p, _d, _p, _d, _p, _p, _d,
                                            _p, _p, _p, _p, _p],
        "oracle_lu_scattering_explicit": [_i, _i, _p, _i, _i, _i, _p, _p, _i, _i, _p, _p, _p, _p],
        "oracle_iterative_system_explicit": [_i, _i, _p, _i, _p, _p, _d, _p],
        "oracle_xgllm": [_i, _i, _i, _i, _i, _p, _p],
        "oracle_t_matrix_element": [_i, _i, _i, _i, _i, _p, _p, _p, _i, _p],
        "oracle_free_propagator_element": [_i, _i, _i, _p, _p, _p, _p, _d, _p, _p, _p, _p],
        "oracle_transition_b_matrix": [_i, _i, _i, _p, _i, _i, _i, _i, _d, _p, _p, _p],
        "oracle_iterative_scattering_explicit": [_i, _i, _i, _p, _i, _i, _i, _p, _p, _i, _i, _p, _p, _d, _d, _p, _p,
                                                 _p],
        "oracle_fms_spectrum_iterative": [_i, _i, _d, _d, _i, _p, _p, _i, _i, _i, _i, _i, _p, _d, _p, _d, _i, _p, _p,
                                          _p, _p, _i],
        "oracle_mkgtr_trace": [_i, _i, _i, _i, _i, _p, _p, _p, _p, _i, _p],
        "oracle_debye_correlation": [_i, _d, _d, _d, _i, _i, _d, _p, _p],
        "oracle_debye_waller": [_i, _d, _d, _d, _i, _p, _p, _p],
        "oracle_debye_sigma2_table": [_i, _i, _p, _p, _i, _p, _d, _d, _d, C.c_float, _p, _p],
        "oracle_fms_lu_system": [_i, _i, _p, _p, _i, _i, _i, _p, _i, _d, _p, _d, _p, _p, _i, _p, _p, _p, _p, _p],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = _i
    L.oracle_legendre_normalization.argtypes = [_i, _i]
    L.oracle_legendre_normalization.restype = _d
    L.oracle_spin_orbit_coefficient.argtypes = [_i, _i, _i, _i]
    L.oracle_spin_orbit_coefficient.restype = _d
    L.oracle_wigner_3j.argtypes = [_i, _i, _i, _i, _i, _i]
    L.oracle_wigner_3j.restype = _d
    L.oracle_wigner_rotation.argtypes = [_d, _i, _i, _i, _i]
    L.oracle_wigner_rotation.restype = _d
    L.oracle_atomic_weight.argtypes = [_i]
    L.oracle_atomic_weight.restype = _d


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_p)


def cbuf(values) -> np.ndarray:
    """Complex array -> interleaved float64 buffer (C-contiguous copy, Fortran order preserved by caller)."""
    a = np.asarray(values, dtype=np.complex128)
    return np.ascontiguousarray(a.reshape(-1, order="F")).view(np.float64).copy()


def from_cbuf(buf: np.ndarray, shape) -> np.ndarray:
    return buf.view(np.complex128).reshape(shape, order="F")


class OracleError(RuntimeError):
    def __init__(self, code: int):
        super().__init__(f"oracle error code {code}")
        self.code = code


def check(rc: int):
    if rc != 0:
        raise OracleError(rc)


def polynomials(lx, lmaxp1, mmaxp1, rho, mode=F32):
    out = np.zeros(2 * (lx + 2) * (2 * lx + 3))
    r = cbuf([rho])
    check(lib().oracle_polynomials(mode, lx, lmaxp1, mmaxp1, ptr(r), ptr(out)))
    return from_cbuf(out, (lx + 2, 2 * lx + 3))


def rotation_matrix(lmax, mmax, beta, phi, forward, mode=F32):
    d = 2 * lmax + 1
    out = np.zeros(2 * d * d * (lmax + 1))
    check(lib().oracle_rotation_matrix(mode, lmax, mmax, float(beta), float(phi), 1 if forward else 0, ptr(out)))
    return from_cbuf(out, (d, d, lmax + 1))


def fms_spectrum(positions, pots, lmaxph, wave_numbers, xphase, *, nsp=1, ispin=0, lfms=0, global_lmax=None,
                 rdirec=1.0e6, sigsqr=None, sig2g=0.0, mode=F64, threads=1):
    """Oracle scattering tables for every energy: array (E, C, C, npot) complex128.

    wave_numbers: (E, nsp) complex; xphase: (E, nsp, 2L+1, npot) complex (FEFF xphase layout per energy).
    """
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    pots = np.ascontiguousarray(pots, dtype=np.int32)
    lmaxph = np.ascontiguousarray(lmaxph, dtype=np.int32)
    npot = len(lmaxph)
    L = int(lmaxph.max()) if global_lmax is None else int(global_lmax)
    E = wave_numbers.shape[0]
    k = cbuf(np.asarray(wave_numbers).reshape(E, nsp).T)  # (nsp, E) F-order == per-energy blocks of nsp
    xp = np.ascontiguousarray(np.asarray(xphase, dtype=np.complex128).reshape(E, -1))
    # per energy: (nsp, 2L+1, npot) column-major
    xp_f = np.stack([np.asarray(xphase[e]).reshape(nsp, 2 * L + 1, npot).reshape(-1, order="F") for e in range(E)])
    xpb = np.ascontiguousarray(xp_f).view(np.float64).copy()
    del xp
    Cc = nsp * (L + 1) ** 2
    out = np.zeros(2 * E * Cc * Cc * npot)
    status = np.zeros(E, dtype=np.int32)
    sig = None if sigsqr is None else np.asfortranarray(sigsqr, dtype=np.float32)
    rc = lib().oracle_fms_spectrum(mode, len(pots), ptr(positions), ptr(pots), nsp, ispin, lfms, npot - 1, L,
                                   ptr(lmaxph), float(rdirec), ptr(sig), float(sig2g), E, ptr(k), ptr(xpb),
                                   ptr(out), ptr(status), int(threads))
    check(rc)
    tabs = out.view(np.complex128).reshape(E, Cc * Cc * npot)
    return np.stack([tabs[e].reshape((Cc, Cc, npot), order="F") for e in range(E)])


def fms_spectrum_iterative(positions, pots, lmaxph, wave_numbers, xphase, *, minv, toler1=1e-3, toler2=1e-3, nsp=1,
                           ispin=0, lfms=0, global_lmax=None, rdirec=1.0e6, sigsqr=None, sig2g=0.0, mode=F64,
                           threads=1, raise_on_error=True):
    """Oracle scattering tables of the iterative forms (minv 1 ggbi, 2 ggrm, 3 gggm, else ggtf): (E, C, C, npot);
    with raise_on_error=False returns (tables, per-energy status)."""
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    pots = np.ascontiguousarray(pots, dtype=np.int32)
    lmaxph = np.ascontiguousarray(lmaxph, dtype=np.int32)
    npot = len(lmaxph)
    L = int(lmaxph.max()) if global_lmax is None else int(global_lmax)
    E = wave_numbers.shape[0]
    k = cbuf(np.asarray(wave_numbers).reshape(E, nsp).T)
    xp_f = np.stack([np.asarray(xphase[e]).reshape(nsp, 2 * L + 1, npot).reshape(-1, order="F") for e in range(E)])
    xpb = np.ascontiguousarray(xp_f).view(np.float64).copy()
    Cc = nsp * (L + 1) ** 2
    out = np.zeros(2 * E * Cc * Cc * npot)
    status = np.zeros(E, dtype=np.int32)
    sig = None if sigsqr is None else np.asfortranarray(sigsqr, dtype=np.float32)
    rc = lib().oracle_fms_spectrum_iterative(mode, int(minv), float(toler1), float(toler2), len(pots), ptr(positions),
                                             ptr(pots), nsp, ispin, lfms, npot - 1, L, ptr(lmaxph), float(rdirec),
                                             ptr(sig), float(sig2g), E, ptr(k), ptr(xpb), ptr(out), ptr(status),
                                             int(threads))
    if raise_on_error:
        check(rc)
    tabs = out.view(np.complex128).reshape(E, Cc * Cc * npot)
    res = np.stack([tabs[e].reshape((Cc, Cc, npot), order="F") for e in range(E)])
    return res if raise_on_error else (res, status)


def iterative_order_spread(positions, pots, lmaxph, wave_numbers, xphase, *, minv, toler1, toler2, mode=F64,
                           permutations=6, seed=0):
    """How far the oracle's own iterative gg moves when the cluster's atoms are listed in another order (the
    representatives of each potential kept in front, the rest shuffled): the same mathematics summed in another
    order.  The FEFF iterative solvers stop on a residual estimate below toler1, so rounding differences move
    their result by up to about toler1 (times the recurrences' amplification); this spread is the scale of any
    faithful reimplementation's disagreement with the oracle.  Returns max |gg' - gg| / max |gg| over the
    absorber block and the energies both runs solved."""
    positions = np.asarray(positions, np.float32)
    pots = np.asarray(pots, np.int32)
    npot = len(lmaxph)
    L = int(np.max(lmaxph))
    m = (L + 1) ** 2
    base, st0 = fms_spectrum_iterative(positions, pots, lmaxph, wave_numbers, xphase, minv=minv, toler1=toler1,
                                       toler2=toler2, mode=mode, raise_on_error=False)
    rng = np.random.default_rng(seed)
    spread = 0.0
    for _ in range(permutations):
        perm = np.concatenate([np.arange(npot), npot + rng.permutation(len(pots) - npot)])
        g, st = fms_spectrum_iterative(positions[perm], pots[perm], lmaxph, wave_numbers, xphase, minv=minv,
                                       toler1=toler1, toler2=toler2, mode=mode, raise_on_error=False)
        ok = [e for e in range(len(st)) if st[e] == 0 and st0[e] == 0]
        if ok:
            ref = np.abs(base[ok, :m, :m, 0]).max()
            spread = max(spread, float(np.abs(g[ok, :m, :m, 0] - base[ok, :m, :m, 0]).max() / ref))
    return spread


def full_scattering(positions, pots, lmaxph, wave_numbers, xphase, *, nsp=1, ispin=0, global_lmax=None,
                    rdirec=1.0e6, sigsqr=None, sig2g=0.0, mode=F64):
    """Oracle save_gg_slice outputs for every energy: the full matrix X = (I - G0 T)^-1 G0 (FmsLuResult's
    full_scattering, crates/refeff-core/src/fms/solvers.rs:473-479, solved with the oracle LU) reduced like
    build_saved_fms_scattering_outputs (crates/refeff-engine/src/fms.rs:4154-4216): slice (E, b, n) = rows [0, b)
    of X over every column, diag (E, N, b, b) = the diagonal block of each atom; b = nsp (L+1)^2, and every atom
    must carry b states (fixed-width atom blocks)."""
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    pots = np.ascontiguousarray(pots, dtype=np.int32)
    lmaxph = np.ascontiguousarray(lmaxph, dtype=np.int32)
    npot, N = len(lmaxph), len(pots)
    L = int(lmaxph.max()) if global_lmax is None else int(global_lmax)
    b = nsp * (L + 1) ** 2
    sig = None if sigsqr is None else np.asfortranarray(sigsqr, dtype=np.float32)
    args = [mode, N, ptr(positions), ptr(pots), nsp, ispin, 0, npot - 1, L, ptr(lmaxph), float(rdirec), ptr(sig),
            float(sig2g)]
    slices, diags = [], []
    for e in range(np.asarray(wave_numbers).shape[0]):
        kb = cbuf(np.asarray(wave_numbers[e]).reshape(nsp))
        xb = cbuf(np.asarray(xphase[e]).reshape(nsp, 2 * L + 1, npot))
        n = np.zeros(1, np.int32)
        check(lib().oracle_fms_energy_intermediates(*args, ptr(kb), ptr(xb), 0.0, ptr(n), None, None, None, None))
        ns = int(n[0])
        if ns != N * b:
            raise ValueError(f"save_gg_slice requires fixed-width atom blocks: {ns} states for {N} atoms of {b}")
        g0, t, a = np.zeros(2 * ns * ns), np.zeros(2 * nsp * ns), np.zeros(2 * ns * ns)
        check(lib().oracle_fms_energy_intermediates(*args, ptr(kb), ptr(xb), 0.0, ptr(n), ptr(g0), ptr(t), ptr(a),
                                                    None))
        _, X, _ = lu_factor_solve(from_cbuf(a, (ns, ns)), from_cbuf(g0, (ns, ns)), mode=mode)
        slices.append(X[:b, :].copy())
        diags.append(np.stack([X[i * b:(i + 1) * b, i * b:(i + 1) * b] for i in range(N)]))
    return np.array(slices), np.array(diags)


def lu_system(positions, pots, lmaxph, wave_number, xphase, *, nsp=1, ispin=0, global_lmax=None, rdirec=1.0e6,
              sigsqr=None, sig2g=0.0, mode=F64, threads=1):
    """The dense system of one energy as the LU form solves it (crates/refeff-core/src/fms/internals/linear.rs:102-135,
    solvers.rs:434-446): returns (A, B, off) with A = I - G0 T (n x n complex128, Fortran order), B = the absorber's
    right-hand sides G0[:, off:off+w] (n x w), so that gg = solve(A, B)[off:off+w, :].  G0 is built on `threads`
    OpenMP threads.  wave_number: (nsp,) complex; xphase: (nsp, 2L+1, npot) complex."""
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    pots = np.ascontiguousarray(pots, dtype=np.int32)
    lmaxph = np.ascontiguousarray(lmaxph, dtype=np.int32)
    npot = len(lmaxph)
    L = int(lmaxph.max()) if global_lmax is None else int(global_lmax)
    kb = cbuf(np.asarray(wave_number).reshape(nsp))
    xb = cbuf(np.asarray(xphase).reshape(nsp, 2 * L + 1, npot))
    sig = None if sigsqr is None else np.asfortranarray(sigsqr, dtype=np.float32)
    n, off, w = (np.zeros(1, np.int64) for _ in range(3))
    args = [mode, len(pots), ptr(positions), ptr(pots), nsp, ispin, L, ptr(lmaxph), npot, float(rdirec), ptr(sig),
            float(sig2g), ptr(kb), ptr(xb), int(threads), ptr(n), ptr(off), ptr(w)]
    check(lib().oracle_fms_lu_system(*args, None, None))
    ns, wd = int(n[0]), int(w[0])
    A = np.zeros((ns, ns), dtype=np.complex128, order="F")
    B = np.zeros((ns, wd), dtype=np.complex128, order="F")
    check(lib().oracle_fms_lu_system(*args, ptr(A), ptr(B)))
    return A, B, int(off[0])


def lu_factor_solve(A, B, mode=F64):
    A = np.asarray(A, dtype=np.complex128)
    B = np.asarray(B, dtype=np.complex128)
    n, m = B.shape
    a = cbuf(A)
    b = cbuf(B)
    piv = np.zeros(n, dtype=np.int64)
    sp = np.zeros(1, dtype=np.int64)
    rc = lib().oracle_lu_factor_solve(mode, n, ptr(a), m, ptr(b), ptr(piv), ptr(sp))
    if rc != 0:
        raise OracleError(rc)
    return from_cbuf(a, (n, n)), from_cbuf(b, (n, m)), piv


def threads_available() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def transition_b_matrix(*, lmax, initial_kappa, polarization, polarization_tensor, multipole, trace_orbital=False,
                        spin=1, spin_channels=1, spin_vector_angle=0.0):
    """FEFF bcoef (crates/refeff-core/src/angular/transition.rs:9-73): returns (bmat, lind, kiind) with bmat of
    shape (2L+1, 2, 8, 2L+1, 2, 8) indexed [m2+L, s2, k2, m1+L, s1, k1] (transitions zero-based)."""
    ML = 2 * lmax + 1
    out = np.zeros(2 * ML * 2 * 8 * ML * 2 * 8)
    ptz = np.ascontiguousarray(np.asarray(polarization_tensor, dtype=np.complex128).reshape(3, 3)).view(np.float64)
    lind = np.zeros(8, np.int32)
    kiind = np.zeros(8, np.int32)
    check(lib().oracle_transition_b_matrix(int(lmax), int(initial_kappa), int(polarization), ptr(ptz),
                                           int(multipole), int(bool(trace_orbital)), int(spin), int(spin_channels),
                                           float(spin_vector_angle), ptr(out), ptr(lind), ptr(kiind)))
    bm = out.view(np.complex128).reshape((ML, 2, 8, ML, 2, 8), order="F")
    return bm, lind, kiind


def mkgtr_trace(gg, bmats, lind, rkk, *, nsp, lmax):
    """getgtr trace (crates/refeff-core/src/fms/mkgtr.rs:790-952): gg (E, dim, dim), bmats list of (2L+1,2,8,2L+1,2,8),
    lind list of 8-int arrays, rkk (E, 8, nsp_rkk) -> traces (nspec, E)."""
    gg = np.asarray(gg, np.complex128)
    E, dim, _ = gg.shape
    g = np.ascontiguousarray(np.stack([gg[e].reshape(-1, order="F") for e in range(E)])).view(np.float64)
    b = np.ascontiguousarray(np.concatenate([np.asarray(x, np.complex128).reshape(-1, order="F") for x in bmats]))
    li = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int32) for x in lind]))
    rk = np.asarray(rkk, np.complex128)
    r = np.ascontiguousarray(rk.reshape(-1, order="F")).view(np.float64)
    nspec = len(bmats)
    out = np.zeros(2 * nspec * E)
    check(lib().oracle_mkgtr_trace(E, dim, int(nsp), int(lmax), nspec, ptr(li), ptr(b.view(np.float64)), ptr(g),
                                   ptr(r), int(rk.shape[2]), ptr(out)))
    return out.view(np.complex128).reshape((nspec, E), order="F")


def atomic_weight(z: int) -> float:
    """FEFF atwtd (crates/refeff-core/src/atomic/tables.rs:10-19): -1.0 outside Z = 1..139."""
    return float(lib().oracle_atomic_weight(int(z)))


def debye_correlation(r, thetad, tk, z1, z2, rsavg, *, classical=False):
    """corrfn / corrfn2 (crates/refeff-core/src/debye/models.rs:88-132): returns (value, romberg iterations)."""
    out = np.zeros(1)
    it = np.zeros(1, np.int32)
    check(lib().oracle_debye_correlation(int(classical), float(r), float(thetad), float(tk), int(z1), int(z2),
                                         float(rsavg), ptr(out), ptr(it)))
    return float(out[0]), int(it[0])


def debye_waller(tk, thetad, rsavg, positions, atomic_numbers, *, classical=False):
    """sigms / sigcl (crates/refeff-core/src/debye/models.rs:134-271) over a path (rows x 3, Angstrom)."""
    pos = np.ascontiguousarray(np.asarray(positions, np.float64).reshape(-1, 3))
    z = np.ascontiguousarray(np.asarray(atomic_numbers, np.int32))
    out = np.zeros(1)
    check(lib().oracle_debye_waller(int(classical), float(tk), float(thetad), float(rsavg), pos.shape[0], ptr(pos),
                                    ptr(z), ptr(out)))
    return float(out[0])


def debye_sigma2_table(idwopt, positions, potentials, atomic_numbers, *, tk, thetad, rsavg, sig2g=0.0):
    """The FMS pair sigma^2 table (crates/refeff-engine/src/fms.rs:4345-4433) for idwopt < 0, 0 or 3: returns
    (table f32 (N, N) indexed [atom2, atom1], Debye term f64 (N, N))."""
    pos = np.ascontiguousarray(np.asarray(positions, np.float32).reshape(-1, 3))
    pots = np.ascontiguousarray(np.asarray(potentials, np.int32))
    z = np.ascontiguousarray(np.asarray(atomic_numbers, np.int32))
    N = pos.shape[0]
    out = np.zeros(N * N, np.float32)
    pair = np.zeros(N * N)
    check(lib().oracle_debye_sigma2_table(int(idwopt), N, ptr(pos), ptr(pots), len(z), ptr(z), float(tk),
                                          float(thetad), float(rsavg), C.c_float(sig2g), ptr(out), ptr(pair)))
    return out.reshape((N, N), order="F"), pair.reshape((N, N), order="F")
