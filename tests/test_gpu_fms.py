"""GPU parity of the FMS path against the CPU oracle, through the C ABI.

Tolerances (relative, Frobenius norm of the absorber block per energy):
  plain FP64 LU           <= 1e-10 versus the FP64 oracle
  FP32 LU + refinement    <= 1e-6  versus the FP64 oracle (the chosen-form gate)
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from refeff_gb300 import fms, workloads as wl

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_CHOSEN = 1e-6


@pytest.fixture(scope="module")
def ctx():
    return fms.Context(0)


def rel_err(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def absorber_blocks(scat, m, abs_pot=0):
    return scat[:, :m, :m, abs_pot]


def run_pair(ctx, cl, grid, form, nsp=1, ispin=0, energies=None, **plan_kw):
    sl = slice(None) if energies is None else energies
    k = grid.wave_numbers[sl]
    ph = grid.phase_shifts[sl]
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph, spin_channels=nsp,
                                   spin_selector=ispin, **plan_kw)
    gpu, status = fms.fms_real_space_spectrum(plan, k, ph, form)
    ref = po.fms_spectrum(cl.positions, cl.potentials, cl.lmaxph, k, ph, nsp=nsp, ispin=ispin, mode=po.F64,
                          threads=po.threads_available(), **{kk: v for kk, v in plan_kw.items()
                                                            if kk in ("rdirec", "sig2g", "sigsqr")})
    return plan, gpu, ref, status


@pytest.mark.parametrize("n,m", [(5, 1), (33, 4), (100, 16), (300, 16)])
def test_dense_lu_fp64_matches_numpy(ctx, n, m):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(3, n, n)) + 1j * rng.normal(size=(3, n, n)) + 4 * np.sqrt(n) * np.eye(n)
    B = rng.normal(size=(3, n, m)) + 1j * rng.normal(size=(3, n, m))
    X, st, _ = fms.complex_lu_solve_batched(ctx, A, B, fms.FORM_FP64_LU)
    assert (st == 0).all()
    for b in range(3):
        assert rel_err(X[b], np.linalg.solve(A[b], B[b])) < 1e-12


def test_dense_lu_fp64_matches_oracle_pivoting(ctx):
    """A matrix that needs row exchanges in every panel (small diagonal)."""
    rng = np.random.default_rng(11)
    n, m = 150, 3
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    A[np.diag_indices(n)] *= 1e-3
    B = rng.normal(size=(n, m)) + 0j
    X, st, _ = fms.complex_lu_solve_batched(ctx, A, B, fms.FORM_FP64_LU)
    _, Xo, _ = po.lu_factor_solve(A, B, po.F64)
    assert st[0] == 0
    assert rel_err(X[0], Xo) < 1e-10


@pytest.mark.parametrize("n", [64, 257, 700, 1100])
def test_dense_lu_fp32_refined(ctx, n):
    rng = np.random.default_rng(n + 1)
    A = rng.normal(size=(2, n, n)) + 1j * rng.normal(size=(2, n, n)) + 3 * np.sqrt(n) * np.eye(n)
    B = rng.normal(size=(2, n, 16)) + 1j * rng.normal(size=(2, n, 16))
    X, st, _ = fms.complex_lu_solve_batched(ctx, A, B, fms.FORM_FP32_REFINED)
    assert (st == 0).all()
    for b in range(2):
        assert rel_err(X[b], np.linalg.solve(A[b], B[b])) < 1e-11


@pytest.mark.parametrize("n,m", [(130, 3), (700, 16), (1100, 25)])
def test_tensor_core_update_matches_cuda_cores(n, m):
    """FP32 LU without refinement: tcgen05 split-TF32 trailing updates against the CUDA-core updates."""
    rng = np.random.default_rng(n + m)
    A = rng.normal(size=(2, n, n)) + 1j * rng.normal(size=(2, n, n)) + 3 * np.sqrt(n) * np.eye(n)
    B = rng.normal(size=(2, n, m)) + 1j * rng.normal(size=(2, n, m))
    out = {}
    for tc in (0, 1):
        c = fms.Context(0)
        c.set_option(c.OPT_TENSOR_CORES, tc)
        c.set_option(c.OPT_DENSE_REFINEMENT, 0)
        out[tc], st, _ = fms.complex_lu_solve_batched(c, A, B, fms.FORM_FP32_REFINED)
        assert (st == 10).all()  # no refinement: flagged NOT_CONVERGED by design
        c.close()
    for b in range(2):
        ref = np.linalg.solve(A[b], B[b])
        assert rel_err(out[0][b], ref) < 1e-5
        assert rel_err(out[1][b], ref) < 1e-5
        assert rel_err(out[1][b], out[0][b]) < 1e-5


@pytest.mark.parametrize("n,m", [(300, 4), (700, 16), (1100, 25)])
def test_paired_blocks_match_single_blocks_with_pivoting(n, m):
    """FP32 LU on the tensor cores with paired 64-column blocks (one K = 128 update per pair, the second block's
    moves applied to the first block's L, its block row corrected by the first block's deferred update) against
    one update per block, on unscaled random systems that pivot in almost every column; without refinement both
    must be FP32-accurate solutions, and with it both must reach the FP64 answer."""
    rng = np.random.default_rng(3 * n + m)
    A = rng.normal(size=(2, n, n)) + 1j * rng.normal(size=(2, n, n))
    B = rng.normal(size=(2, n, m)) + 1j * rng.normal(size=(2, n, m))
    ref = [np.linalg.solve(A[b], B[b]) for b in range(2)]
    raw, refined = {}, {}
    for paired in (0, 1):
        c = fms.Context(0)
        c.set_option(c.OPT_PAIRED_BLOCKS, paired)
        c.set_option(c.OPT_DENSE_REFINEMENT, 0)
        raw[paired], st, _ = fms.complex_lu_solve_batched(c, A, B, fms.FORM_FP32_REFINED)
        assert (st == 10).all()
        c.set_option(c.OPT_DENSE_REFINEMENT, 10)
        refined[paired], st, _ = fms.complex_lu_solve_batched(c, A, B, fms.FORM_FP32_REFINED)
        assert (st == 0).all()
        c.close()
    for b in range(2):
        # complex64 LAPACK reaches ~1e-6 on these systems (condition numbers 4e2 - 4e3); the split-TF32 products
        # keep 22 of FP32's 24 bits and the block rows use the explicit L11^-1, so the GPU's unrefined FP32
        # solutions land near 1e-4 (measured 1.7e-4 at n = 700); a wrong row order or a missed deferred update
        # gives O(1) errors
        assert rel_err(raw[0][b], ref[b]) < 2e-3
        assert rel_err(raw[1][b], ref[b]) < 2e-3
        assert rel_err(raw[1][b], raw[0][b]) < 2e-3
        assert rel_err(refined[1][b], ref[b]) < 1e-10
        assert rel_err(refined[0][b], ref[b]) < 1e-10


def test_dense_lu_singular_reports_pivot(ctx):
    n = 40
    rng = np.random.default_rng(5)
    A = rng.normal(size=(n, n)) + 0j
    A[:, 7] = 0.0  # exactly singular: a zero column
    B = np.ones((n, 2), np.complex128)
    X, st, piv = fms.complex_lu_solve_batched(ctx, A, B, fms.FORM_FP64_LU)
    assert st[0] == 9  # SingularMatrix
    assert piv[0] == 8  # 1-based first zero pivot
    assert np.isfinite(X).all()


def test_fms_small_cluster_fp64(ctx):
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=6)
    plan, gpu, ref, status = run_pair(ctx, cl, grid, fms.FORM_FP64_LU)
    assert (status == 0).all()
    m = plan.shape.absorber_block
    assert np.count_nonzero(gpu[:, m:, :, :]) == 0 and np.count_nonzero(gpu[:, :, m:, :]) == 0
    assert np.count_nonzero(gpu[:, :, :, 1]) == 0  # only the absorber potential is solved (lfms = 0)
    for e in range(gpu.shape[0]):
        assert rel_err(gpu[e], ref[e]) < TOL_FP64, e


@pytest.mark.parametrize("form,tol", [(fms.FORM_FP64_LU, TOL_FP64), (fms.FORM_FP32_REFINED, 1e-6),
                                      (fms.FORM_BICGSTAB, 1e-6)])
def test_fms_all_potentials_lfms(ctx, form, tol):
    """lfms != 0: every potential's representative block is solved (fms_lu_scattering over the whole potential
    range, solvers.rs:434-471): a two-potential cluster with lmaxph [3, 2] (right-hand sides 16 + 9) and the
    three-potential rocksalt cluster (16 + 16 + 16), against the FP64 oracle."""
    cases = []
    cl, grid = wl.small_cluster(3.0, lmax=3, n_energies=4, seed=17)
    cl.lmaxph = np.array([3, 2], np.int32)
    cases.append((cl, grid))
    rs = wl.rocksalt_cluster(np.random.default_rng(5), radius=4.6)
    cases.append((rs, wl.energy_grid(rs, 4, 10.0, 60.0, seed=5)))
    for cl, grid in cases:
        plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph, lfms=1)
        gpu, status = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts, form)
        assert (status == 0).all()
        ref = po.fms_spectrum(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers, grid.phase_shifts,
                              lfms=1, mode=po.F64, threads=po.threads_available())
        npot = len(cl.lmaxph)
        for e in range(gpu.shape[0]):
            for q in range(npot):
                assert np.abs(ref[e, :, :, q]).max() > 0, q
                assert rel_err(gpu[e, :, :, q], ref[e, :, :, q]) < tol, (e, q)


def test_full_scattering_save_gg_slice(ctx):
    """save_gg_slice: the full matrix X = (I - G0 T)^-1 G0 (solvers.rs:473-479) reduced to the absorber's rows over
    every column and each atom's diagonal block (engine/fms.rs:4154-4216), FP64 LU against the oracle's own LU
    of the same system, for lfms 0 (n = 117) and lfms 1 (n = 304, all potentials); the full plan's scattering
    table equals an ordinary plan's, and the absorber's diagonal block is its absorber block."""
    cases = [(*wl.small_cluster(3.0, lmax=2, n_energies=3, seed=3), {}),
             (*wl.small_cluster(3.7, lmax=3, n_energies=2, seed=4), {"lfms": 1})]
    for cl, grid, kw in cases:
        plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph, full_scattering=True, **kw)
        tab, sl, dg, st = fms.fms_full_scattering_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
        assert (st == 0).all()
        ref_sl, ref_dg = po.full_scattering(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers,
                                            grid.phase_shifts)
        b, n, N = plan.shape.channel_count, plan.shape.n_states, cl.n_atoms
        assert sl.shape == ref_sl.shape == (len(st), b, n) and dg.shape == ref_dg.shape == (len(st), N, b, b)
        for e in range(len(st)):
            assert rel_err(sl[e], ref_sl[e]) < TOL_FP64, e
            assert rel_err(dg[e], ref_dg[e]) < TOL_FP64, e
        assert np.array_equal(sl[:, :, :b], dg[:, 0])
        plain = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph, **kw)
        tab2, _ = fms.fms_real_space_spectrum(plain, grid.wave_numbers, grid.phase_shifts)
        assert rel_err(tab, tab2) < 1e-12
        for e in range(len(st)):
            assert rel_err(dg[e, 0], tab[e, :, :, 0]) < 1e-12


def test_full_scattering_plan_rules(ctx):
    """Atoms of different widths are refused (fixed-width atom blocks, engine/fms.rs:4164-4172); the request
    forces the LU form (driver.rs:72-96): minv is dropped and only the FP64 LU form is accepted; an ordinary plan
    has no full-scattering output."""
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=2, seed=8)
    with pytest.raises(fms.FmsError) as e:
        fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, [2, 1], full_scattering=True)
    assert e.value.code == 13 and "fixed-width" in str(e.value)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph, full_scattering=True, minv=1)
    with pytest.raises(fms.FmsError) as e:
        fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts, fms.FORM_FP32_REFINED)
    assert e.value.code == 1
    tab, _, _, st = fms.fms_full_scattering_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
    lu = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    tab2, _ = fms.fms_real_space_spectrum(lu, grid.wave_numbers, grid.phase_shifts)
    assert (st == 0).all() and rel_err(tab, tab2) < 1e-12
    with pytest.raises(fms.FmsError) as e:
        fms.fms_full_scattering_spectrum(lu, grid.wave_numbers, grid.phase_shifts)
    assert e.value.code == 1


def test_fms_small_cluster_fp32_refined(ctx):
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=6)
    plan, gpu, ref, status = run_pair(ctx, cl, grid, fms.FORM_FP32_REFINED)
    assert (status == 0).all()
    for e in range(gpu.shape[0]):
        assert rel_err(gpu[e], ref[e]) < TOL_CHOSEN, e


def test_fms_config0_subset_both_forms(ctx):
    """fcc Cu <= 4.5 A (43 atoms, n = 688): 8 energies across the grid."""
    cl, grid = wl.config0()
    sel = np.linspace(0, 99, 8).astype(int)
    plan, gpu64, ref, st64 = run_pair(ctx, cl, grid, fms.FORM_FP64_LU, energies=sel)
    assert plan.shape.n_states == 688 and plan.shape.absorber_block == 16
    gpu32, st32 = fms.fms_real_space_spectrum(plan, grid.wave_numbers[sel], grid.phase_shifts[sel],
                                              fms.FORM_FP32_REFINED)
    assert (st64 == 0).all() and (st32 == 0).all()
    for e in range(len(sel)):
        assert rel_err(gpu64[e], ref[e]) < TOL_FP64, e
        assert rel_err(gpu32[e], ref[e]) < TOL_CHOSEN, e


def test_fms_config1_sample_against_oracle(ctx):
    """fcc Cu <= 7.5 A (141 atoms, n = 2256, two-level cluster panels): 16 of the 200 energies against the FP64
    oracle, weighted to the low end of the grid where k is smallest and the systems are worst conditioned."""
    cl, grid = wl.config1()
    sel = np.array([0, 1, 2, 3, 4, 6, 9, 14, 22, 36, 60, 90, 120, 150, 175, 199])
    plan, gpu64, ref, st64 = run_pair(ctx, cl, grid, fms.FORM_FP64_LU, energies=sel)
    assert plan.shape.n_states == 2256
    gpu32, st32 = fms.fms_real_space_spectrum(plan, grid.wave_numbers[sel], grid.phase_shifts[sel],
                                              fms.FORM_FP32_REFINED)
    assert (st64 == 0).all() and (st32 == 0).all()
    for e in range(len(sel)):
        assert rel_err(gpu64[e], ref[e]) < TOL_FP64, e
        assert rel_err(gpu32[e], ref[e]) < TOL_CHOSEN, e


def test_refinement_stats_and_fallback(ctx):
    """An unattainable tolerance forces every energy through the FP64 fallback; results stay at the FP64 bar."""
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=3, seed=21)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    ok, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts, fms.FORM_FP32_REFINED)
    rel, its, fb = plan.refinement_stats(3)
    assert (fb == 0).all() and (its >= 1).all() and (rel < 1e-4).all()
    plan.set_refinement(1, 1e-300)
    forced, st = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts, fms.FORM_FP32_REFINED)
    rel, its, fb = plan.refinement_stats(3)
    assert (fb == 1).all() and (st == 0).all()
    ref64, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts, fms.FORM_FP64_LU)
    assert rel_err(forced, ref64) < 1e-15


def test_fms_reference_precision_agreement(ctx):
    """The reference computes in Complex32: the f32-faithful oracle sits within f32 error of the GPU FP64 path."""
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=4, seed=3)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    gpu, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
    f32 = po.fms_spectrum(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers, grid.phase_shifts, mode=po.F32)
    for e in range(gpu.shape[0]):
        assert rel_err(gpu[e], f32[e]) < 1e-3


def test_fms_spin_orbit_two_spins(ctx):
    """nsp = 2 with distinct j = l -/+ 1/2 phase shifts: compact T with the spin-flip partner band."""
    cl, grid = wl.small_cluster(2.6, lmax=2, n_energies=3, seed=9, nsp=2)
    rng = np.random.default_rng(1)
    ph = grid.phase_shifts.copy()
    L = cl.global_lmax
    ph[:, :, :L, :] *= 1.0 + 0.2 * rng.random(ph[:, :, :L, :].shape)  # -l slots differ from +l
    ph[:, 1] *= 0.9
    grid.phase_shifts = ph
    plan, gpu, ref, status = run_pair(ctx, cl, grid, fms.FORM_FP64_LU, nsp=2)
    assert (status == 0).all()
    for e in range(gpu.shape[0]):
        assert rel_err(gpu[e], ref[e]) < TOL_FP64, e


def test_fms_spin_selector_one_spin(ctx):
    cl, grid = wl.small_cluster(2.6, lmax=2, n_energies=3, seed=10)
    ph = grid.phase_shifts.copy()
    ph[:, :, :cl.global_lmax, :] *= 0.8
    grid.phase_shifts = ph
    plan, gpu, ref, status = run_pair(ctx, cl, grid, fms.FORM_FP64_LU, ispin=1)
    assert (status == 0).all()
    for e in range(gpu.shape[0]):
        assert rel_err(gpu[e], ref[e]) < TOL_FP64, e


def test_fms_debye_damping_and_cutoff(ctx):
    cl, grid = wl.small_cluster(3.7, lmax=2, n_energies=3, seed=12)
    plan, gpu, ref, status = run_pair(ctx, cl, grid, fms.FORM_FP64_LU, direct_cutoff=3.0, sig2g=0.004)
    ref2 = po.fms_spectrum(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers, grid.phase_shifts,
                           rdirec=3.0, sig2g=0.004, mode=po.F64)
    for e in range(gpu.shape[0]):
        assert rel_err(gpu[e], ref2[e]) < TOL_FP64, e


def test_fms_nonfinite_phase_flags_only_that_energy(ctx):
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=4, seed=13)
    ph = grid.phase_shifts.copy()
    ph[2, 0, cl.global_lmax + 1, 1] = np.nan
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    gpu, status = fms.fms_real_space_spectrum(plan, grid.wave_numbers, ph, raise_on_error=False)
    assert status[2] == 6 and (status[[0, 1, 3]] == 0).all()
    ref = po.fms_spectrum(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers[[0, 1, 3]],
                          grid.phase_shifts[[0, 1, 3]], mode=po.F64)
    for i, e in enumerate([0, 1, 3]):
        assert rel_err(gpu[e], ref[i]) < TOL_FP64


def test_fms_batching_is_invariant(ctx):
    """Results do not depend on how energies are split into device batches (graph replay included)."""
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=11, seed=14)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    full, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
    plan.set_batch(4)
    split, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
    again, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
    assert np.array_equal(split, again)
    assert rel_err(split, full) < 1e-13


@pytest.mark.parametrize("form", [fms.FORM_FP64_LU, fms.FORM_FP32_REFINED])
def test_fms_calls_of_different_sizes_on_one_plan(ctx, form):
    """A plan called with few energies, then many, then few again returns what fresh plans return: a CUDA
    graph captured for one batch size is never replayed for another."""
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=9, seed=15)
    k, ph = grid.wave_numbers, grid.phase_shifts
    fresh = {}
    for E in (2, 9):
        p0 = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
        fresh[E], _ = fms.fms_real_space_spectrum(p0, k[:E], ph[:E], form)
        p0.close()
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    for E in (2, 2, 9, 9, 2):
        got, st = fms.fms_real_space_spectrum(plan, k[:E], ph[:E], form)
        assert (st == 0).all()
        assert rel_err(got, fresh[E]) < 1e-12, E


def test_device_pointer_entry_point(ctx):
    torch = pytest.importorskip("torch")
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=5, seed=15)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    host, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
    E, m = 5, plan.shape.absorber_block
    L, npot = cl.global_lmax, len(cl.lmaxph)
    k = torch.from_numpy(np.ascontiguousarray(grid.wave_numbers)).cuda()
    xp = np.ascontiguousarray(np.stack([grid.phase_shifts[e].reshape(-1, order="F") for e in range(E)]))
    x = torch.from_numpy(xp).cuda()
    gg = torch.zeros((E, m * m), dtype=torch.complex128, device="cuda")
    st = torch.zeros(E, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    fms.fms_real_space_spectrum_device(plan, k.data_ptr(), x.data_ptr(), E, gg.data_ptr(), st.data_ptr())
    torch.cuda.synchronize()
    dev = gg.cpu().numpy().reshape(E, m, m).transpose(0, 2, 1)  # column-major blocks
    assert (st.cpu().numpy() == 0).all()
    assert rel_err(dev, host[:, :m, :m, 0]) < 1e-14


def test_gg_section_pads_to_output_spin_capacity(ctx):
    cl, grid = wl.small_cluster(2.6, lmax=2, n_energies=1, seed=16)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    scat, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
    sec = fms.gg_section(plan, scat[0], nspu=2)
    m = plan.shape.absorber_block
    assert sec.shape == (2 * m, 2 * m)
    assert np.array_equal(sec[:m, :m], scat[0, :m, :m, 0])
    assert np.abs(sec[m:, :]).max() == 0 and np.abs(sec[:, m:]).max() == 0


@pytest.mark.parametrize("form", [fms.FORM_FP32_REFINED, fms.FORM_FP64_LU])
def test_two_stream_batches_give_identical_results(form):
    """Two-stream batching (REFEFF_FMS_OPT_DUAL_STREAMS: batches alternate between two workspaces on two
    streams) computes every energy with the same kernels on the same inputs, so its results equal the
    one-stream run bit for bit; 20 energies in batches of 5 exercise both workspaces and the join."""
    cl, grid = wl.config0()
    sel = np.arange(0, 100, 5)
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    out = {}
    for dual in (0, 1):
        c = fms.Context(0)
        c.set_option(c.OPT_DUAL_STREAMS, dual)
        plan = fms.fms_real_space_plan(c, cl.positions, cl.potentials, cl.lmaxph)
        plan.set_batch(5)
        out[dual], st = fms.fms_real_space_spectrum(plan, k, ph, form)
        assert (st == 0).all()
        again, _ = fms.fms_real_space_spectrum(plan, k, ph, form)   # graph replay on both streams
        assert np.array_equal(again, out[dual])
        plan.close()
        c.close()
    assert np.array_equal(out[0], out[1])
