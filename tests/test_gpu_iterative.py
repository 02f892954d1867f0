"""FEFF iterative FMS forms (minv 1 ggbi, 2 ggrm, 3 gggm, 4 ggtf) on the GPU against the oracle's
restatement (itself pinned to the reference's solver known answers, crates/refeff-core/src/fms/tests/solvers.rs).

These solvers stop once a residual estimate falls below toler1, and their recurrences amplify rounding: the
oracle run on the same cluster with the atoms listed in another order (same mathematics, other summation
order) already moves gg by up to ~1e-3 of max|gg| for gggm / ggtf at toler1 = 1e-3, ~4e-6 for ggrm, and
~1e-16 for the single-step ggbi (tests/test_oracle_properties.py shows that this spread follows toler1).
The GPU keeps the absorber last, so its tolerances are set from that spread: ggbi 1e-9 (FP64) / 1e-5 (FP32);
the others 1e-6 at toler1 = 1e-7, where all of them are converged, and at the reference default
toler1 = 1e-3 30x the spread measured on the same case and arithmetic (pyoracle.iterative_order_spread),
capped at 1e-2.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from refeff_gb300 import fms
from refeff_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return fms.Context(0)


def _case(lmax=2, n_energies=4, seed=5, nsp=1, radius=2.6):
    return wl.small_cluster(radius, lmax=lmax, n_energies=n_energies, seed=seed, nsp=nsp)


def _gpu(ctx, cl, grid, minv, form, toler1, toler2, nsp=1, ispin=0):
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph, minv=minv, spin_channels=nsp,
                                   spin_selector=ispin, convergence_tolerance=toler1, zero_tolerance=toler2)
    scat, st = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts, form, raise_on_error=False)
    return scat, st, plan.shape.absorber_block


TOL64 = {1: (1.0e-3, 1.0e-9), 2: (1.0e-7, 1.0e-6), 3: (1.0e-7, 1.0e-6), 4: (1.0e-7, 1.0e-6)}


def _rel(g, w, m):
    return np.abs(g[:, :m, :m, 0] - w[:, :m, :m, 0]).max() / np.abs(w[:, :m, :m, 0]).max()


def _spread_gate(cl, grid, minv, toler1, toler2, mode):
    """30x the oracle's own atom-order spread on this case, at most 1e-2 and at least 1e-9."""
    spread = po.iterative_order_spread(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers, grid.phase_shifts,
                                       minv=minv, toler1=toler1, toler2=toler2, mode=mode)
    return min(1e-2, max(30.0 * spread, 1e-9))


@pytest.mark.parametrize("minv", [1, 2, 3, 4])
@pytest.mark.parametrize("toler2", [0.0, 1.0e-3])
def test_iterative_fp64_matches_oracle(ctx, minv, toler2):
    cl, grid = _case()
    toler1, bound = TOL64[minv]
    scat, st, m = _gpu(ctx, cl, grid, minv, fms.FORM_FP64_LU, toler1, toler2)
    want, ost = po.fms_spectrum_iterative(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers,
                                          grid.phase_shifts, minv=minv, toler1=toler1, toler2=toler2, mode=po.F64,
                                          raise_on_error=False)
    assert list(st) == [0] * len(st) and list(ost) == [0] * len(ost)
    assert _rel(scat, want, m) <= bound


@pytest.mark.parametrize("minv", [1, 2, 3, 4])
def test_iterative_all_potentials_lfms(ctx, minv):
    """lfms != 0: every potential's representative states are sources (iterative.rs:98-171), here lmaxph [2, 1]
    (blocks of 9 and 4 states), both forms against the oracle's all-potential iterative run."""
    cl, grid = _case(seed=13)
    lmaxph = np.array([2, 1], np.int32)
    toler1, bound = TOL64[minv]
    for form, mode, t1, bnd in [(fms.FORM_FP64_LU, po.F64, toler1, bound),
                                (fms.FORM_FP32_REFINED, po.F32, 1.0e-3, 1e-5 if minv == 1 else 1e-2)]:
        plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, lmaxph, minv=minv, lfms=1,
                                       convergence_tolerance=t1, zero_tolerance=0.0)
        scat, st = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts, form,
                                               raise_on_error=False)
        want, ost = po.fms_spectrum_iterative(cl.positions, cl.potentials, lmaxph, grid.wave_numbers,
                                              grid.phase_shifts, minv=minv, toler1=t1, toler2=0.0, lfms=1,
                                              mode=mode, raise_on_error=False)
        both = [e for e in range(len(st)) if st[e] == 0 and ost[e] == 0]
        assert len(both) >= len(st) // 2 and all(v in (0, 19) for v in st)
        for q, ip in enumerate((9, 4)):
            g, w = scat[both][:, :ip, :ip, q], want[both][:, :ip, :ip, q]
            assert np.abs(w).max() > 0
            assert np.abs(g - w).max() <= bnd * np.abs(w).max(), (form, q)


@pytest.mark.parametrize("minv", [2, 3, 4])
def test_iterative_fp64_at_reference_tolerance(ctx, minv):
    cl, grid = _case(seed=9)
    scat, st, m = _gpu(ctx, cl, grid, minv, fms.FORM_FP64_LU, 1.0e-3, 1.0e-3)
    want = po.fms_spectrum_iterative(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers, grid.phase_shifts,
                                     minv=minv, toler1=1.0e-3, toler2=1.0e-3, mode=po.F64)
    assert list(st) == [0] * len(st)
    assert _rel(scat, want, m) <= _spread_gate(cl, grid, minv, 1.0e-3, 1.0e-3, po.F64)


@pytest.mark.parametrize("minv", [1, 2, 3, 4])
def test_iterative_fp32_matches_reference_precision_oracle(ctx, minv):
    cl, grid = _case(seed=9)
    scat, st, m = _gpu(ctx, cl, grid, minv, fms.FORM_FP32_REFINED, 1.0e-3, 1.0e-3)
    want, ost = po.fms_spectrum_iterative(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers,
                                          grid.phase_shifts, minv=minv, toler1=1.0e-3, toler2=1.0e-3, mode=po.F32,
                                          raise_on_error=False)
    # Complex32 gggm breaks down at some energies in the reference arithmetic (a zero divisor); compare the
    # energies both sides solved and require the GPU to report 0 or the breakdown code elsewhere.
    both = [e for e in range(len(st)) if st[e] == 0 and ost[e] == 0]
    assert len(both) >= len(st) // 2
    assert all(st[e] in (0, 19) for e in range(len(st)))
    bound = 1e-5 if minv == 1 else _spread_gate(cl, grid, minv, 1.0e-3, 1.0e-3, po.F32)
    assert _rel(scat[both], want[both], m) <= bound


@pytest.mark.parametrize("minv", [1, 4])
def test_iterative_spin_orbit_partner_terms(ctx, minv):
    cl, grid = _case(lmax=2, n_energies=3, seed=12, nsp=2)
    toler1, bound = TOL64[minv]
    scat, st, m = _gpu(ctx, cl, grid, minv, fms.FORM_FP64_LU, toler1, 0.0, nsp=2)
    want = po.fms_spectrum_iterative(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers, grid.phase_shifts,
                                     minv=minv, toler1=toler1, toler2=0.0, nsp=2, mode=po.F64)
    assert list(st) == [0] * len(st)
    assert _rel(scat, want, m) <= bound


def test_converging_forms_approach_the_lu_solution(ctx):
    cl, grid = _case(seed=21)
    lu, _, m = _gpu(ctx, cl, grid, 0, fms.FORM_FP64_LU, 1.0e-3, 0.0)
    ref = np.abs(lu[:, :m, :m, 0]).max()
    for minv in (2, 3, 4):
        it, st, _ = _gpu(ctx, cl, grid, minv, fms.FORM_FP64_LU, 1.0e-7, 0.0)
        assert list(st) == [0] * len(st)
        assert np.abs(it[:, :m, :m, 0] - lu[:, :m, :m, 0]).max() <= 1e-4 * ref, minv


def test_recursion_without_tolerance_reports_no_convergence(ctx):
    cl, grid = _case(lmax=1, n_energies=2, seed=2)
    _, st, _ = _gpu(ctx, cl, grid, 2, fms.FORM_FP64_LU, 0.0, 0.0)
    _, ost = po.fms_spectrum_iterative(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers, grid.phase_shifts,
                                       minv=2, toler1=0.0, toler2=0.0, mode=po.F64, raise_on_error=False)
    assert list(st) == [10] * len(st)
    assert all(v == -13 for v in ost)
