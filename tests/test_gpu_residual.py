"""The refinement residual on the tensor cores against the double-float residual on the FP32 pipes.

r = b - A x of the FP32 LU forms is computed, by default, from exact products of 8-bit digits of A (scaled per
row over 32-column segments) and of x (scaled per column) on the bf16 tensor path, the exact level sums combined
in double-float, one pass per 16 right-hand sides (REFEFF_FMS_OPT_RESIDUAL_TENSOR = 1); option 0 runs the Dot2
residual on the CUDA cores.  Both
must carry the FP32 LU to the FP64 answer: on dense systems whose entries span many orders of magnitude inside
each row (so the segment scales differ along a row) with right-hand sides of unequal size, on column counts that
leave the 16-column slots partly empty, on orders that leave the last 128-row tile and the last 32-column segment
ragged, and on FMS systems.  A residual whose bounded wait gives up sends the call to the FP64 LU.
"""
import numpy as np
import pytest

from refeff_gb300 import fms, workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fms.Context(0)
    yield c
    c.close()


def rel_err(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def _dense_case(n, m, seed):
    rng = np.random.default_rng(seed)
    mag = 10.0 ** rng.uniform(-6, 0, size=(2, n, n))
    A = (rng.normal(size=(2, n, n)) + 1j * rng.normal(size=(2, n, n))) * mag + 3 * np.sqrt(n) * np.eye(n)
    A *= 10.0 ** rng.uniform(-2, 2, size=(2, n, 1))                       # row scales
    X = (rng.normal(size=(2, n, m)) + 1j * rng.normal(size=(2, n, m))) * 10.0 ** rng.uniform(-1, 1, size=(2, 1, m))
    X *= 10.0 ** rng.uniform(-8, 0, size=(2, n, m))                          # tiny entries inside each column
    return A, A @ X


@pytest.mark.parametrize("n,m", [(64, 1), (200, 9), (333, 13), (688, 16), (1100, 16), (700, 25), (300, 32)])
def test_tensor_residual_refines_to_fp64(n, m):
    A, B = _dense_case(n, m, 13 * n + m)
    out = {}
    for flag in (1, 0):
        c = fms.Context(0)
        c.set_option(c.OPT_RESIDUAL_TENSOR, flag)
        out[flag], st, _ = fms.complex_lu_solve_batched(c, A, B, fms.FORM_FP32_REFINED)
        c.close()
        assert (st == 0).all(), (flag, st)
    for b in range(2):
        ref = np.linalg.solve(A[b], B[b])
        assert rel_err(out[1][b], ref) < 1e-10, b
        assert rel_err(out[0][b], ref) < 1e-10, b
        assert rel_err(out[1][b], out[0][b]) < 1e-10, b


def test_tensor_residual_fms_matches_dot2(ctx):
    """fcc Cu <= 4.5 A (n = 688, 16 absorber columns): both residuals reach the FP64 LU's gg with the same number
    of corrections, give or take one."""
    cl, grid = wl.config0()
    sel = np.array([0, 5, 17, 40, 66, 99])
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    m = plan.shape.absorber_block
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    g64, s64 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    assert (s64 == 0).all()
    res = {}
    try:
        for flag in (1, 0):
            ctx.set_option(ctx.OPT_RESIDUAL_TENSOR, flag)
            g, st = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP32_REFINED)
            assert (st == 0).all(), (flag, st)
            rel, its, fb = plan.refinement_stats(len(sel))
            assert not fb.any(), (flag, fb)
            res[flag] = (g, its)
    finally:
        ctx.set_option(ctx.OPT_RESIDUAL_TENSOR, 1)
    for e in range(len(sel)):
        ref = g64[e, :m, :m, 0]
        assert rel_err(res[1][0][e, :m, :m, 0], ref) < 1e-9, e
        assert rel_err(res[0][0][e, :m, :m, 0], ref) < 1e-9, e
        assert abs(int(res[1][1][e]) - int(res[0][1][e])) <= 1, (e, res[1][1], res[0][1])
    plan.close()


def test_tensor_residual_wait_timeout_falls_back_to_fp64_lu():
    """The BiCGSTAB form runs no tensor-core LU update before its first residual, so with a one-poll budget the
    residual's own waits give up: the kernel raises the error flag, drains its copies and MMAs, frees its tensor
    memory, and the call is solved again by the FP64 LU (the refined-LU stage times out the same way)."""
    ctx = fms.Context(0)
    cl, grid = wl.config0()
    sel = np.array([40, 66, 99])
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    m = plan.shape.absorber_block
    g64, s64 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    assert (s64 == 0).all()
    try:
        ctx.set_option(fms.Context.OPT_TC_WAIT_POLLS, 1)
        gb, sb = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
        msg = ctx.last_error()
    finally:
        ctx.set_option(fms.Context.OPT_TC_WAIT_POLLS, 0)
    assert "timed out" in msg, msg
    assert (sb == 0).all(), sb
    _, _, fallback = plan.refinement_stats(len(sel))
    assert fallback.all(), fallback
    for e in range(len(sel)):
        assert rel_err(gb[e, :m, :m, 0], g64[e, :m, :m, 0]) < 1e-13, e
    # default budget again: the BiCGSTAB form completes on its own
    gb2, sb2 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_BICGSTAB)
    assert (sb2 == 0).all()
    for e in range(len(sel)):
        assert rel_err(gb2[e, :m, :m, 0], g64[e, :m, :m, 0]) < 1e-6, e
    plan.close()
    ctx.close()
