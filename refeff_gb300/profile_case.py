"""Small, repeatable FMS workload for profilers (ncu): one named configuration,
a given number of energies, one form, two sweeps (the first one captures the
CUDA graph).

    python -m refeff_gb300.profile_case --config 1 --energies 16 --form fp32
"""
from __future__ import annotations

import argparse

from . import fms, workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=1, choices=[0, 1])
    ap.add_argument("--energies", type=int, default=16)
    ap.add_argument("--form", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--sweeps", type=int, default=2)
    args = ap.parse_args()
    cl, grid = (workloads.config0 if args.config == 0 else workloads.config1)()
    E = args.energies
    form = fms.FORM_FP32_REFINED if args.form == "fp32" else fms.FORM_FP64_LU
    ctx = fms.Context(0)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    plan.set_batch(E)
    for _ in range(args.sweeps):
        _, status = fms.fms_real_space_spectrum(plan, grid.wave_numbers[:E], grid.phase_shifts[:E], form)
    print("ok", int((status != 0).sum()), "failed energies")


if __name__ == "__main__":
    main()
