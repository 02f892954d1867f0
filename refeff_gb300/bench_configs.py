"""Throughput of every solver form on the batched, learned and large configurations.

    python -m refeff_gb300.bench_configs --config 2|3|4 [--energies E] [--fp64-energies E64]

Prints one JSON line per configuration: energy points/s of the plain FP64 LU, the FP32 LU + FP64
refinement, and (configurations 3 and 4) the BiCGSTAB form without and with the learned preconditioner,
each timed with CUDA-synchronised wall clocks through the host-buffer entry point, on an evenly spaced
sample of the configuration's energies (the FP64 LU on a smaller sub-sample, the same energies for its
comparison), plus the largest relative gg error of each chosen form against the FP64 LU.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import fms, learned, workloads


def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def _rel(a, b, m):
    return float(max(np.linalg.norm(a[e, :m, :m, 0] - b[e, :m, :m, 0]) /
                     max(np.linalg.norm(b[e, :m, :m, 0]), 1e-300) for e in range(a.shape[0])))


def single_cluster(ctx, cl, grid, n_energies, n_fp64, forms, model=None):
    E_all = grid.wave_numbers.shape[0]
    sel = np.unique(np.linspace(0, E_all - 1, n_energies).round().astype(int))
    sub = sel[np.unique(np.linspace(0, len(sel) - 1, n_fp64).round().astype(int))]
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    m = plan.shape.absorber_block
    out = {"n": plan.shape.n_states, "m": m, "energies": int(len(sel)), "fp64_energies": int(len(sub))}
    (g64, _), t64 = _timed(lambda: fms.fms_real_space_spectrum(plan, grid.wave_numbers[sub], grid.phase_shifts[sub],
                                                               fms.FORM_FP64_LU))
    out["fp64_lu"] = {"points_per_s": len(sub) / t64}
    pos = {int(e): i for i, e in enumerate(sel)}
    idx = np.array([pos[int(e)] for e in sub])
    for name, form, mdl in forms:
        plan.set_preconditioner(model if mdl else None)
        fms.fms_real_space_spectrum(plan, grid.wave_numbers[sel[:2]], grid.phase_shifts[sel[:2]], form)  # warm
        (g, st), t = _timed(lambda: fms.fms_real_space_spectrum(plan, grid.wave_numbers[sel], grid.phase_shifts[sel],
                                                                form, raise_on_error=False))
        rec = {"points_per_s": len(sel) / t, "over_fp64": (len(sel) / t) / out["fp64_lu"]["points_per_s"],
               "max_rel_gg_err_vs_fp64": _rel(g[idx], g64, m), "status_nonzero": int((st != 0).sum())}
        _, _, fb = plan.refinement_stats(len(sel))
        rec["fp64_fallbacks"] = int(fb.sum())
        if form == fms.FORM_BICGSTAB:
            its = plan.bicgstab_stats(len(sel))
            rec["bicgstab_iterations_mean"] = float(its.mean())
        out[name] = rec
    plan.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, required=True, choices=[2, 3, 4])
    ap.add_argument("--energies", type=int, default=0, help="sampled energies (0: the configuration's default)")
    ap.add_argument("--fp64-energies", type=int, default=0)
    ap.add_argument("--train-cases", type=int, default=8)
    args = ap.parse_args()
    ctx = fms.Context(0)
    if args.config == 2:
        cases = workloads.config2()
        plans = [fms.fms_real_space_plan(ctx, c.positions, c.potentials, c.lmaxph) for c, _ in cases]
        ks = [g.wave_numbers for _, g in cases]
        phs = [g.phase_shifts for _, g in cases]
        res = {"config": 2, "workload": "32 seeded displaced fcc clusters, 150 energies each, one call",
               "energy_points": int(sum(len(k) for k in ks))}
        for name, form in (("fp64_lu", fms.FORM_FP64_LU), ("fp32_refined", fms.FORM_FP32_REFINED)):
            fms.fms_real_space_spectrum_multi(plans, [k[:2] for k in ks], [p[:2] for p in phs], form)
            (tabs, sts), t = _timed(lambda: fms.fms_real_space_spectrum_multi(plans, ks, phs, form))
            res[name] = {"points_per_s": res["energy_points"] / t, "seconds": t,
                         "status_nonzero": int(sum(int((s != 0).sum()) for s in sts))}
            res[name + "_tables"] = tabs
        t64, t32 = res.pop("fp64_lu_tables"), res.pop("fp32_refined_tables")
        res["fp32_refined"]["over_fp64"] = res["fp32_refined"]["points_per_s"] / res["fp64_lu"]["points_per_s"]
        res["fp32_refined"]["max_rel_gg_err_vs_fp64"] = max(
            _rel(a, b, p.shape.absorber_block) for a, b, p in zip(t32, t64, plans))
        print(json.dumps(res), flush=True)
        return
    if args.config == 3:
        cl, grid = workloads.config3()
        n_e, n64 = args.energies or 60, args.fp64_energies or 12
        t0 = time.perf_counter()
        train = learned.rocksalt_training_cases(args.train_cases, radius_range=(6.0, 8.0), n_energies=300, seed=11,
                                                material_seed=3)
        X, T = learned.training_set(ctx, train, energies_per_case=25, atoms_per_case=10, seed=5)
        model, hist = learned.train_preconditioner(ctx, 3, X, T, hidden=96, epochs=800, batch_size=256,
                                                   learning_rate=1e-3, seed=6)
        train_s = time.perf_counter() - t0
        forms = [("fp32_refined", fms.FORM_FP32_REFINED, False), ("bicgstab", fms.FORM_BICGSTAB, False),
                 ("bicgstab_learned", fms.FORM_BICGSTAB, True)]
        res = single_cluster(ctx, cl, grid, n_e, n64, forms, model)
        res.update({"config": 3, "workload": "rocksalt AB a=4.44 A, sigma 0.04 A, R 9 A, lmax 3, 300 energies",
                    "training": {"fp64_lu_solves": int(X.shape[0]), "clusters": args.train_cases,
                                 "loss_first": float(hist[0]), "loss_last": float(hist[-1]), "seconds": train_s}})
        print(json.dumps(res), flush=True)
        return
    cl, grid = workloads.config4()
    n_e, n64 = args.energies or 8, args.fp64_energies or 2
    forms = [("fp32_refined", fms.FORM_FP32_REFINED, False), ("bicgstab", fms.FORM_BICGSTAB, False)]
    res = single_cluster(ctx, cl, grid, n_e, n64, forms)
    res.update({"config": 4, "workload": "random close packed 600 atoms, lmax 4 (n = 15000), 400 energies"})
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
