"""BiCGSTAB form and its learned diagonal preconditioner.

CPU: the network's CPU restatement (oracle/mlp_oracle.py) against finite differences.
GPU: the training kernels' loss and gradient against that restatement; the feature kernel against its
restatement; the FP64-LU training targets against a dense inverse; the BiCGSTAB form against the FP64 LU
(<= 1e-6, the chosen-form gate); and what the trained network gains: fewer BiCGSTAB iterations than the
unpreconditioned solve on held-out clusters and energies.  Block Jacobi with per-atom blocks is the identity
here (the same-atom blocks of G0 vanish, so every diagonal block of I - G0 T is I), so the unpreconditioned
solve is also the block-Jacobi baseline.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo
from oracle import pyoracle as po
from refeff_gb300 import fms, learned, workloads as wl


def _random_problem(rng, F=7, H=5, O=4, S=9):
    n = H * F + H + H * H + H + O * H + O
    return rng.normal(size=n) * 0.4, rng.normal(size=(S, F)), rng.normal(size=(S, O)) * 0.3


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    F, H, O = 7, 5, 4
    p, X, T = _random_problem(rng, F, H, O)
    _, g = mo.loss_grad(p, F, H, O, X, T)
    eps = 1e-6
    for i in rng.choice(p.size, size=40, replace=False):
        dp = np.zeros_like(p)
        dp[i] = eps
        num = (mo.loss_grad(p + dp, F, H, O, X, T)[0] - mo.loss_grad(p - dp, F, H, O, X, T)[0]) / (2 * eps)
        assert abs(num - g[i]) <= 1e-7 + 1e-6 * abs(num), i


def test_feature_and_output_counts():
    assert mo.feature_count(3) == 40 and mo.output_count(3) == 32
    assert mo.feature_count(4) == 48 and mo.output_count(4) == 50
    assert mo.output_count(3, 1) == 2 * 16 * 16 and mo.output_count(2, 1) == 2 * 81


def test_oracle_block_preconditioner_layout():
    """Row-major Re/Im layout: output 2 (q C + q2) is Re B[q, q2]; channels beyond an atom's lmax are zero, and
    energies outside the window get the identity."""
    L, c = 1, 4
    Y = np.zeros((2, 2, 2 * c * c))
    Y[:, :, 2 * (0 * c + 1)] = 0.5       # Re B[0, 1]
    Y[:, :, 2 * (1 * c + 0) + 1] = -0.25  # Im B[1, 0]
    Y[:, :, 2 * (3 * c + 3)] = 9.0       # B[3, 3]: beyond lmax 0 for atom 1
    B = mo.block_preconditioner(Y, [1, 0], L, [True, False])
    assert B[0, 0, 0, 1] == 0.5 and B[0, 0, 1, 0] == -0.25j and B[0, 0, 3, 3] == 10.0
    assert B[0, 1, 0, 0] == 1.0 and np.count_nonzero(B[0, 1]) == 1
    assert np.array_equal(B[1, 0], np.eye(c)) and np.count_nonzero(B[1, 1]) == 1


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def ctx():
    return fms.Context(0)


@pytest.mark.gpu
def test_gpu_loss_and_gradient_match_oracle(ctx):
    rng = np.random.default_rng(1)
    model = fms.PrecondModel(ctx, 2, hidden=24, seed=3)
    F, H, O = model.n_features, model.hidden, model.n_outputs
    p = (rng.normal(size=model.n_params) * 0.3).astype(np.float32)
    model.set_params(p)
    X = rng.normal(size=(300, F)).astype(np.float32)
    T = (rng.normal(size=(300, O)) * 0.2).astype(np.float32)
    loss, g = model.loss_grad(X, T)
    ref_loss, ref_g = mo.loss_grad(p.astype(np.float64), F, H, O, X, T)
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss
    assert np.linalg.norm(g - ref_g) <= 1e-4 * np.linalg.norm(ref_g)
    Y = model.predict(X)
    assert np.abs(Y - mo.forward(p, F, H, O, X)[2]).max() <= 1e-4


@pytest.mark.gpu
def test_gpu_training_reduces_loss(ctx):
    rng = np.random.default_rng(2)
    model = fms.PrecondModel(ctx, 1, hidden=32, seed=5)
    X = rng.normal(size=(2048, model.n_features)).astype(np.float32)
    T = np.tanh(X[:, :model.n_outputs] * 0.7 + 0.2 * X[:, 1:2]).astype(np.float32)
    hist = model.train(X, T, epochs=60, batch_size=128, learning_rate=3e-3, seed=1)
    assert hist[-1] < 0.2 * hist[0]
    assert np.all(np.isfinite(hist))


@pytest.mark.gpu
def test_gpu_features_match_oracle(ctx):
    cl, grid = wl.small_cluster(4.0, lmax=3, n_energies=5, seed=2)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    F = mo.feature_count(3)
    got = plan.precond_features(grid.wave_numbers, grid.phase_shifts, F)
    N = cl.n_atoms
    order = [learned.device_index(a, N) for a in range(N)]
    pos_dev = np.zeros((N, 3))
    pot_dev = np.zeros(N, int)
    for a in range(N):
        pos_dev[order[a]] = cl.positions[a]
        pot_dev[order[a]] = cl.potentials[a]
    want = mo.features(grid.wave_numbers, grid.phase_shifts, pos_dev, pot_dev, 3, len(cl.lmaxph))
    assert np.abs(got - want).max() <= 2e-5 * max(1.0, np.abs(want).max())


@pytest.mark.gpu
def test_gpu_inverse_diagonal_matches_dense_inverse(ctx):
    """Training targets from the FP64 LU = the diagonal of a dense inverse of the oracle's system matrix."""
    import sys
    sys.path.insert(0, str(__import__("pathlib").Path(__file__).parent))
    from test_oracle_properties import _intermediates
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=3, seed=9)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    b = 9
    for atom in (0, 1, cl.n_atoms - 1):
        diag, st = plan.inverse_diagonal(grid.wave_numbers, grid.phase_shifts, atom)
        assert (st == 0).all() and diag.shape == (3, b)
        for e in range(3):
            _, _, A = _intermediates(cl, grid.wave_numbers[e], grid.phase_shifts[e])
            inv = np.linalg.inv(A)
            ref = np.diag(inv)[atom * b:(atom + 1) * b]
            assert np.abs(diag[e] - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.gpu
def test_gpu_inverse_block_matches_dense_inverse(ctx):
    """Block-model targets from the FP64 LU = the atom's whole block of a dense inverse; its diagonal is the
    diagonal target."""
    import sys
    sys.path.insert(0, str(__import__("pathlib").Path(__file__).parent))
    from test_oracle_properties import _intermediates
    cl, grid = wl.small_cluster(3.0, lmax=2, n_energies=3, seed=9)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    b = 9
    for atom in (0, 2, cl.n_atoms - 1):
        blk, st = plan.inverse_block(grid.wave_numbers, grid.phase_shifts, atom)
        diag, _ = plan.inverse_diagonal(grid.wave_numbers, grid.phase_shifts, atom)
        assert (st == 0).all() and blk.shape == (3, b, b)
        assert np.array_equal(np.diagonal(blk, axis1=1, axis2=2), diag)
        for e in range(3):
            _, _, A = _intermediates(cl, grid.wave_numbers[e], grid.phase_shifts[e])
            ref = np.linalg.inv(A)[atom * b:(atom + 1) * b, atom * b:(atom + 1) * b]
            assert np.abs(blk[e] - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.gpu
def test_gpu_untrained_block_model_is_the_identity(ctx):
    """A fresh block model (zero last layer) applies exact identity blocks: the BiCGSTAB form gives the same
    iterations and bit-identical blocks as the unpreconditioned solve; a non-zero model still meets 1e-6."""
    cl, grid = wl.config0()
    sel = np.arange(50, 100, 9)
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    g0, st0 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    it0 = plan.bicgstab_stats(len(sel))
    model = fms.PrecondModel(ctx, plan.inputs["L"], hidden=16, seed=2, kind=fms.PRECOND_BLOCK)
    assert model.n_outputs == mo.output_count(plan.inputs["L"], 1)
    plan.set_preconditioner(model)
    g1, st1 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    it1 = plan.bicgstab_stats(len(sel))
    assert (st0 == 0).all() and (st1 == 0).all()
    assert np.array_equal(it0, it1)
    assert np.array_equal(g0, g1)
    p = model.params()
    rng = np.random.default_rng(4)
    p[-model.n_outputs * (model.hidden + 1):] = rng.normal(size=model.n_outputs * (model.hidden + 1)) * 0.002
    model.set_params(p)
    g2, st2 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    g64, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    assert (st2 == 0).all()
    m = plan.shape.absorber_block
    for e in range(len(sel)):
        ref = g64[e, :m, :m, 0]
        assert np.linalg.norm(g2[e, :m, :m, 0] - ref) <= 1e-6 * np.linalg.norm(ref), e
    plan.set_preconditioner(None)
    model.close()


@pytest.mark.gpu
def test_gpu_bicgstab_form_matches_fp64_lu(ctx):
    cl, grid = wl.config0()
    sel = np.arange(50, 100, 7)      # the energies above the edge, where BiCGSTAB converges
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    g64, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    gb, st = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    assert (st == 0).all()
    its = plan.bicgstab_stats(len(sel))
    assert (its > 0).all()
    m = plan.shape.absorber_block
    for e in range(len(sel)):
        ref = g64[e, :m, :m, 0]
        assert np.linalg.norm(gb[e, :m, :m, 0] - ref) <= 1e-6 * np.linalg.norm(ref), e


@pytest.mark.gpu
@pytest.mark.parametrize("lmax,mode", [(3, 1), (4, 1), (3, 2), (4, 2)])
def test_gpu_bicgstab_tensor_product_matches_cuda_cores(ctx, lmax, mode):
    """The BiCGSTAB form with its matrix-vector products on the tensor cores (split TF32, four products (mode 1)
    or three (mode 2); 16 accumulator columns at lmax 3, 32 at lmax 4 for the 25 right-hand sides) and on the
    FP32 CUDA cores: both meet the 1e-6 gate
    against the FP64 LU with every energy solved by BiCGSTAB (no product gave up), in about the same number of
    iterations."""
    cl, grid = wl.small_cluster(6.0, lmax=lmax, n_energies=12, seed=5)
    sel = np.arange(6, 12)  # 17..40 eV: every energy converges within the 400-iteration cap
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    g64, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    m = plan.shape.absorber_block
    its = {}
    try:
        for tensor in (mode, 0):
            ctx.set_option(ctx.OPT_BICG_TENSOR, tensor)
            g, st = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
            its[tensor] = plan.bicgstab_stats(len(sel))
            assert (st == 0).all() and (plan.bicgstab_lu_energies(len(sel)) == 0).all(), tensor
            for e in range(len(sel)):
                ref = g64[e, :m, :m, 0]
                assert np.linalg.norm(g[e, :m, :m, 0] - ref) <= 1e-6 * np.linalg.norm(ref), (tensor, e)
    finally:
        ctx.set_option(ctx.OPT_BICG_TENSOR, 1)
    print("iterations, tensor cores (mode %d) vs CUDA cores:" % mode, its[mode].sum(), its[0].sum())
    assert abs(int(its[mode].sum()) - int(its[0].sum())) <= 0.25 * its[0].sum()


@pytest.mark.gpu
def test_gpu_bicgstab_iteration_cap_falls_back_to_lu(ctx):
    """A cap of 3 iterations misses the tolerance: those energies are re-solved by the refined LU (FP32
    factorisation + FP64 refinement) and flagged; no FP64 fallback is needed."""
    cl, grid = wl.config0()
    sel = np.array([60, 80])
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    plan.set_bicgstab(max_iterations=3, tolerance=1e-6, poll_interval=1)
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    g64, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    g32, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP32_REFINED)
    gb, st = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    assert (st == 0).all()
    assert (plan.bicgstab_lu_energies(len(sel)) == 1).all()
    _, _, fb = plan.refinement_stats(len(sel))
    assert not fb.any()
    m = plan.shape.absorber_block
    ref = g64[:, :m, :m, 0]
    assert np.linalg.norm(gb[:, :m, :m, 0] - ref) <= 1e-9 * np.linalg.norm(ref)
    assert np.linalg.norm(gb - g32) <= 1e-12 * np.linalg.norm(g32)


@pytest.mark.gpu
def test_gpu_bicgstab_window_routes_energies_to_the_refined_lu(ctx):
    """Energies outside the BiCGSTAB window are not iterated (0 iterations, flag 2) and come from the refined
    LU; the energies inside are the same BiCGSTAB solves as without a window."""
    cl, grid = wl.config0()
    sel = np.arange(40, 100, 6)
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    e_ev = 0.5 * (k[:, 0].real ** 2 - k[:, 0].imag ** 2) * 0.529177249 ** 2 * 27.211396
    srt = np.sort(e_ev)
    lo, hi = 0.5 * (srt[2] + srt[3]), 0.5 * (srt[7] + srt[8])  # midway: no energy on an edge
    inside = (e_ev >= lo) & (e_ev <= hi)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    g64, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    gall, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    itall = plan.bicgstab_stats(len(sel))
    plan.set_bicgstab_window(lo, hi)
    gw, st = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    itw = plan.bicgstab_stats(len(sel))
    flags = plan.bicgstab_lu_energies(len(sel))
    assert (st == 0).all()
    assert (flags[~inside] == 2).all() and (itw[~inside] == 0).all()
    assert (itw[inside] > 0).all()
    ok = inside & (flags == 0)
    assert np.array_equal(itw[ok], itall[ok])
    m = plan.shape.absorber_block
    for e in range(len(sel)):
        ref = g64[e, :m, :m, 0]
        assert np.linalg.norm(gw[e, :m, :m, 0] - ref) <= 1e-6 * np.linalg.norm(ref), e


@pytest.mark.gpu
def test_gpu_learned_preconditioner_reduces_iterations(ctx):
    """Train on FP64-LU targets from seeded rocksalt clusters (radius 4.5-5.5 A, one material), then solve a
    held-out geometry of the same material: the learned diagonal needs fewer BiCGSTAB iterations than none, at
    the same accuracy."""
    train = learned.rocksalt_training_cases(4, radius_range=(4.5, 5.5), n_energies=120, seed=21)
    X, T = learned.training_set(ctx, train, energies_per_case=40, atoms_per_case=12, seed=3,
                                energy_window=(-10.0, 100.0))
    model, hist = learned.train_preconditioner(ctx, 3, X, T, hidden=96, epochs=800, batch_size=128,
                                               learning_rate=1e-3, seed=4)
    assert hist[-1] < 0.5 * hist[0]
    held = wl.rocksalt_cluster(np.random.default_rng(99), radius=5.2)
    grid = wl.energy_grid(held, 120, -20.0, 100.0, seed=3)  # the training material
    sel = np.where((grid.energies_ev > -8.0) & (grid.energies_ev < 30.0))[0][::4]
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    plan = fms.fms_real_space_plan(ctx, held.positions, held.potentials, held.lmaxph)
    plan.set_bicgstab(max_iterations=2000, tolerance=1e-6, poll_interval=16)
    g64, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    g0, st0 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    it0 = plan.bicgstab_stats(len(sel))
    plan.set_preconditioner(model)
    g1, st1 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    it1 = plan.bicgstab_stats(len(sel))
    assert (st0 == 0).all() and (st1 == 0).all()
    m = plan.shape.absorber_block
    for g in (g0, g1):
        for e in range(len(sel)):
            ref = g64[e, :m, :m, 0]
            assert np.linalg.norm(g[e, :m, :m, 0] - ref) <= 1e-6 * np.linalg.norm(ref)
    print("BiCGSTAB iterations, none vs learned:", it0.sum(), it1.sum())
    assert it1.sum() < 0.9 * it0.sum()


@pytest.mark.gpu
def test_gpu_learned_block_preconditioner_meets_the_gate(ctx):
    """The block model on the same training material: whole per-atom blocks of A^-1 as targets, trained on the
    GPU; on a held-out geometry the BiCGSTAB form with it meets the 1e-6 gate with no energy handed to the LU.
    (It is not asserted to beat the diagonal model: the exact per-atom blocks of A^-1 precondition worse than
    their diagonal on these clusters, 782 against 604 iterations at -7.9 eV on the R = 5.2 A cluster.)"""
    train = learned.rocksalt_training_cases(4, radius_range=(4.5, 5.5), n_energies=120, seed=21)
    X, T = learned.training_set(ctx, train, energies_per_case=40, atoms_per_case=12, seed=3,
                                energy_window=(-10.0, 100.0), kind=fms.PRECOND_BLOCK)
    assert T.shape[1] == mo.output_count(3, 1)
    model, hist = learned.train_preconditioner(ctx, 3, X, T, hidden=96, epochs=800, batch_size=128,
                                               learning_rate=1e-3, seed=4, kind=fms.PRECOND_BLOCK)
    assert hist[-1] < 0.5 * hist[0]
    held = wl.rocksalt_cluster(np.random.default_rng(99), radius=5.2)
    grid = wl.energy_grid(held, 120, -20.0, 100.0, seed=3)
    sel = np.where((grid.energies_ev > -8.0) & (grid.energies_ev < 30.0))[0][::4]
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    plan = fms.fms_real_space_plan(ctx, held.positions, held.potentials, held.lmaxph)
    plan.set_bicgstab(max_iterations=2000, tolerance=1e-6, poll_interval=16)
    g64, _ = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    it0 = plan.bicgstab_stats(len(sel))
    plan.set_preconditioner(model)
    g1, st1 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    it1 = plan.bicgstab_stats(len(sel))
    assert (st1 == 0).all() and (plan.bicgstab_lu_energies(len(sel)) == 0).all()
    m = plan.shape.absorber_block
    for e in range(len(sel)):
        ref = g64[e, :m, :m, 0]
        assert np.linalg.norm(g1[e, :m, :m, 0] - ref) <= 1e-6 * np.linalg.norm(ref)
    print("BiCGSTAB iterations, none vs learned block:", it0.sum(), it1.sum())
