"""The large configurations on the GPU, pinned to the FP64 oracle.

config 3 (rocksalt, 257 atoms, n = 4112) and config 4 (random close packing, 600 atoms, lmax 4, n = 15000) exercise
the 16-column inner panels, the panel bookkeeping in global memory, 8-column FP64 panels and the blocked
(unfused) triangular sweeps, which the smaller clusters do not reach.

Oracle pin: for a few energies the oracle builds the dense system itself, A = I - G0 T and the absorber's
right-hand sides B = G0[:, absorber] in FP64 (oracle/fms_oracle.cpp, restating
crates/refeff-core/src/fms/internals/linear.rs:102-135 and solvers.rs:366-484), and the host solves it with an
independent FP64 LU, LAPACK's zgetrf/zgetrs as bundled with scipy.  The GPU's plain FP64 LU must match that
absorber block within 1e-10 relative (Frobenius) and the chosen FP32 + refinement form within 1e-6.  The oracle's
own unblocked LU takes minutes per energy at these sizes, LAPACK's blocked LU seconds.

Beyond the pinned energies, the refined FP32 form is checked against the GPU's FP64 LU (the size-independent
property that both forms agree within the chosen-form gate).
"""
import numpy as np
import pytest

from refeff_gb300 import fms, workloads as wl

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_CHOSEN = 1e-6


def oracle_absorber_block(cl, grid, e):
    """gg of energy e from the oracle's FP64 system solved by LAPACK (scipy), reference state order."""
    sl = pytest.importorskip("scipy.linalg")
    from oracle import pyoracle as po
    A, B, off = po.lu_system(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers[e], grid.phase_shifts[e],
                             threads=po.threads_available())
    lu = sl.lu_factor(A, overwrite_a=True, check_finite=False)
    del A
    X = sl.lu_solve(lu, B, check_finite=False)
    w = B.shape[1]
    return X[off:off + w, :]


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
    # the lowest energy (smallest k) and the middle of the grid against the oracle's system
    for i in (0, 1):
        ref = oracle_absorber_block(cl, grid, sel[i])
        assert ref.shape == (m, m)
        assert rel_err(g64[i, :m, :m, 0], ref) < TOL_FP64, i
        assert rel_err(g32[i, :m, :m, 0], ref) < TOL_CHOSEN, i


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
    # the lowest energy against the oracle's system (n = 15000: 3.6 GB in FP64 on the host)
    ref = oracle_absorber_block(cl, grid, sel[0])
    assert ref.shape == (m, m)
    assert rel_err(g64[0, :m, :m, 0], ref) < TOL_FP64
    assert rel_err(g32[0, :m, :m, 0], ref) < TOL_CHOSEN


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


def test_repeated_many_cluster_call_runs_as_one_graph():
    """A repeated many-cluster call with the same plans, energies and form is captured once as one CUDA graph and
    replayed: every call gives bit-identical tables (the graph holds the same kernels as the per-plan launch
    sequences), a plan setting between calls retires the graph (no replay with stale arguments), and the option
    switches it off."""
    ctx = fms.Context(0)
    cases = wl.config2()[::4]
    sel = np.array([0, 75, 149])
    plans = [fms.fms_real_space_plan(ctx, c.positions, c.potentials, c.lmaxph) for c, _ in cases]
    ks = [g.wave_numbers[sel] for _, g in cases]
    phs = [g.phase_shifts[sel] for _, g in cases]
    runs = []
    for _ in range(4):
        tables, sts = fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP32_REFINED)
        assert all((s == 0).all() for s in sts)
        runs.append(tables)
    assert ctx.graph_stats() == (1, 2)  # plain, capture + launch, two replays
    for t in runs[1:]:
        assert all(np.array_equal(a, b) for a, b in zip(t, runs[0]))
    plans[0].set_tuning(16, -1)  # a setting the graph bakes in: the next call may not replay
    t5, _ = fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP32_REFINED)
    assert ctx.graph_stats()[1] == 2
    plans[0].set_tuning(0, -1)
    ref64, _ = fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP64_LU)
    for p, a, r in zip(plans, t5, ref64):
        m = p.shape.absorber_block
        assert rel_err(a[:, :m, :m, 0], r[:, :m, :m, 0]) < TOL_CHOSEN
    # a plan's buffers grown by a larger single-plan call in between: the next repeat may not replay the graph
    # (it holds the old pointers); it runs the per-plan launch sequences and the repeat after that recaptures
    for _ in range(2):
        fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP32_REFINED)
    cap0, rep0 = ctx.graph_stats()
    big = np.arange(0, 150, 10)
    fms.fms_real_space_spectrum(plans[1], cases[1][1].wave_numbers[big], cases[1][1].phase_shifts[big],
                                fms.FORM_FP32_REFINED)
    t6, _ = fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP32_REFINED)
    assert ctx.graph_stats()[1] == rep0
    assert all(np.array_equal(a, b) for a, b in zip(t6, runs[0]))
    ctx.set_option(ctx.OPT_MULTI_GRAPH, 0)
    for _ in range(3):
        t, _ = fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP32_REFINED)
        assert all(np.array_equal(a, b) for a, b in zip(t, runs[0]))
    assert ctx.graph_stats()[1] == rep0
    for p in plans:
        p.close()
    ctx.close()


def test_autotuned_many_cluster_call_matches_default(ctx, tmp_path):
    """The batched form's autotuner (per size bucket: inner panel width and block pairing; then the stream count)
    on 10 of config 2's clusters with a 4-energy sample: the tuned many-cluster call gives the default call's
    results (both within the chosen-form gate of the FP64 LU), the choice is written to the JSON cache, and a
    second call with the same workload applies it from the cache without measuring."""
    import json
    cases = wl.config2()[::3]
    sel = np.array([0, 40, 80, 120, 149])
    plans = [fms.fms_real_space_plan(ctx, c.positions, c.potentials, c.lmaxph) for c, _ in cases]
    ks = [g.wave_numbers[sel] for _, g in cases]
    phs = [g.phase_shifts[sel] for _, g in cases]
    ref64, _ = fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP64_LU)
    before, _ = fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP32_REFINED)
    cache = tmp_path / "autotune.json"
    got = fms.autotune_multi(plans, ks, phs, fms.FORM_FP32_REFINED, sample_energies=4, cache_path=cache)
    assert not got["from_cache"] and got["streams"] in (2, 4, 8, 16) and got["buckets"] >= 2
    assert got["seconds_tuned"] <= got["seconds_default"] * 1.5
    entries = json.loads(cache.read_text())["entries"]
    assert len(entries) == 1 and next(iter(entries.values()))["streams"] == got["streams"]
    after, sts = fms.fms_real_space_spectrum_multi(plans, ks, phs, fms.FORM_FP32_REFINED)
    assert all((s == 0).all() for s in sts)
    for p, a, b, r in zip(plans, after, before, ref64):
        m = p.shape.absorber_block
        assert rel_err(a[:, :m, :m, 0], r[:, :m, :m, 0]) < TOL_CHOSEN
        assert rel_err(b[:, :m, :m, 0], r[:, :m, :m, 0]) < TOL_CHOSEN
    for p in plans:
        p.set_tuning(0, -1)
    again = fms.autotune_multi(plans, ks, phs, fms.FORM_FP32_REFINED, sample_energies=4, cache_path=cache)
    assert again["from_cache"] and again["streams"] == got["streams"]
    for p in plans:
        p.close()
