"""The tensor-core update's bounded waits, made to run out on purpose.

Every mbarrier wait between the roles of the tcgen05 trailing update (copy producer, MMA issuer, epilogue
groups) is bounded by a poll budget, a context option.  With a budget of one poll, waits give up long before
their copies or MMAs land.  The kernel then sets its error flag, ends every role, waits with the full default
budget for the copies and MMAs it has in flight (so nothing is outstanding when a CTA exits) and frees its
tensor memory.  The host reads the flag after the call and solves every energy of the call again with the
plain FP64 LU.  Nothing faults: the wait is bounded, not broken.

Checked here: the call succeeds with every status 0, its results equal the FP64 LU form's, the context's last
error names the timeout, and with the default budget restored the same plan solves normally again.
"""
import numpy as np
import pytest

from refeff_gb300 import fms, workloads as wl

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_tensor_core_wait_timeout_falls_back_to_fp64_lu():
    ctx = fms.Context(0)
    cl, grid = wl.config0()
    sel = np.array([0, 33, 66, 99])
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    m = plan.shape.absorber_block
    assert plan.shape.n_states == 688          # large enough for the tensor-core trailing update
    g64, s64 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    assert (s64 == 0).all()
    try:
        ctx.set_option(fms.Context.OPT_TC_WAIT_POLLS, 1)
        g32, s32 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP32_REFINED)
        msg = ctx.last_error()
    finally:
        ctx.set_option(fms.Context.OPT_TC_WAIT_POLLS, 0)
    assert "timed out" in msg, msg
    assert (s32 == 0).all(), s32
    _, _, fallback = plan.refinement_stats(len(sel))
    assert fallback.all(), fallback            # every energy of the call went to the FP64 LU
    for e in range(len(sel)):
        assert rel_err(g32[e, :m, :m, 0], g64[e, :m, :m, 0]) < 1e-13, e
    # default budget again: the tensor-core path completes and meets the chosen-form gate on its own
    g32b, s32b = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP32_REFINED)
    assert (s32b == 0).all()
    _, _, fallback_b = plan.refinement_stats(len(sel))
    assert not fallback_b.any(), fallback_b
    for e in range(len(sel)):
        assert rel_err(g32b[e, :m, :m, 0], g64[e, :m, :m, 0]) < 1e-6, e
    plan.close()
    ctx.close()
