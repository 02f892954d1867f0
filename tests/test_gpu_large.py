"""The large configurations on the GPU, beyond the oracle's reach at full size.

config 3 (rocksalt, 257 atoms, n = 4112) and config 4 (random close packing, 600 atoms, lmax 4, n = 15000) exercise
the 16-column inner panels, the panel bookkeeping in global memory, 8-column FP64 panels and the blocked
(unfused) triangular sweeps.  Full-size oracle runs take minutes per energy here, so these tests check the
size-independent property that the refined FP32 form agrees with the plain FP64 LU (itself pinned to the
oracle at smaller sizes) within the chosen-form gate 1e-6.
"""
import numpy as np
import pytest

from refeff_gb300 import fms, workloads as wl

pytestmark = pytest.mark.gpu

TOL_CHOSEN = 1e-6


@pytest.fixture(scope="module")
def ctx():
    return fms.Context(0)


def rel_err(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _two_forms(ctx, cl, grid, sel):
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    plan.set_batch(len(sel))
    k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
    g64, s64 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP64_LU)
    g32, s32 = fms.fms_real_space_spectrum(plan, k, ph, fms.FORM_FP32_REFINED)
    return plan, g64, s64, g32, s32


def test_config3_rocksalt_refined_matches_fp64(ctx):
    cl, grid = wl.config3()
    sel = np.array([0, 150, 299])
    plan, g64, s64, g32, s32 = _two_forms(ctx, cl, grid, sel)
    m = plan.shape.absorber_block
    assert plan.shape.n_states == 4112 and m == 16
    assert (s64 == 0).all() and (s32 == 0).all()
    for e in range(len(sel)):
        assert rel_err(g32[e, :m, :m, 0], g64[e, :m, :m, 0]) < TOL_CHOSEN, e


def test_config4_n15000_refined_matches_fp64(ctx):
    cl, grid = wl.config4()
    sel = np.array([0, 399])
    plan, g64, s64, g32, s32 = _two_forms(ctx, cl, grid, sel)
    m = plan.shape.absorber_block
    assert plan.shape.n_states == 15000 and m == 25
    assert (s64 == 0).all() and (s32 == 0).all()
    for e in range(len(sel)):
        blk = g64[e, :m, :m, 0]
        assert np.abs(blk).max() > 0
        assert rel_err(g32[e, :m, :m, 0], blk) < TOL_CHOSEN, e


def test_config2_many_clusters_in_one_call(ctx):
    """config 2: 32 seeded displaced fcc clusters (n from 9*43 to 16*141), 150 energies each; here every
    cluster with 4 energies through one multi-cluster call, checked against one call per plan (same kernels,
    so equal to rounding) and the smallest clusters against the FP64 oracle."""
    from oracle import pyoracle as po
    cases = wl.config2()
    sel = np.array([0, 50, 100, 149])
    plans = [fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph) for cl, _ in cases]
    ks = [g.wave_numbers[sel] for _, g in cases]
    phs = [g.phase_shifts[sel] for _, g in cases]
    for form, tol in ((fms.FORM_FP64_LU, 1e-10), (fms.FORM_FP32_REFINED, 1e-6)):
        tables, sts = fms.fms_real_space_spectrum_multi(plans, ks, phs, form)
        assert all((s == 0).all() for s in sts)
        for i in (0, 13, 31):
            single, _ = fms.fms_real_space_spectrum(plans[i], ks[i], phs[i], form)
            m = plans[i].shape.absorber_block
            assert rel_err(tables[i][:, :m, :m, 0], single[:, :m, :m, 0]) < 1e-12
        small = sorted(range(len(cases)), key=lambda i: plans[i].shape.n_states)[:2]
        for i in small:
            cl, _ = cases[i]
            ref = po.fms_spectrum(cl.positions, cl.potentials, cl.lmaxph, ks[i], phs[i], mode=po.F64,
                                  threads=po.threads_available())
            m = plans[i].shape.absorber_block
            for e in range(len(sel)):
                assert rel_err(tables[i][e, :m, :m, 0], ref[e, :m, :m, 0]) < tol, (i, e)
