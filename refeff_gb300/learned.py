"""Training workflow of the learned BiCGSTAB preconditioner.

The targets come from the FP64 LU path itself: for sampled (cluster, energy,
atom) the diagonal of the atom's block of (I - G0 T)^-1
(refeff_fms_plan_inverse_diagonal), paired with the features the GPU computes
for that atom (refeff_fms_plan_precond_features).  The network is trained on the
GPU (refeff_fms_precond_train) and attached to a plan for the BiCGSTAB form.
"""
from __future__ import annotations

import numpy as np

from . import fms, workloads


def device_index(atom: int, n_atoms: int) -> int:
    """Device atom order keeps the reference order with the absorber moved last."""
    return n_atoms - 1 if atom == 0 else atom - 1


def training_set(ctx: fms.Context, cases, *, energies_per_case: int, atoms_per_case: int, seed: int = 0,
                 energy_window=None, kind: int = fms.PRECOND_DIAGONAL):
    """(X, T): features and targets of sampled atoms and energies.

    Targets: diag(block of A^-1) - 1, Re/Im per channel (kind PRECOND_DIAGONAL), or the whole block of A^-1
    minus the identity, row-major C x C (C = (L+1)^2), Re/Im interleaved, zero beyond the atom's own channels
    (PRECOND_BLOCK, one spin channel).  cases: list of (Cluster, EnergyGrid); energy_window: optional (lo, hi)
    in eV on the grid's energies."""
    rng = np.random.default_rng(seed)
    Xs, Ts = [], []
    for cl, grid in cases:
        plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
        L = plan.inputs["L"]
        Cc = (L + 1) ** 2
        F, O = 2 + 2 * (L + 1) + 3 * (2 + 2 * (L + 1)), (2 * Cc * Cc if kind == fms.PRECOND_BLOCK else 2 * Cc)
        idx = np.arange(grid.wave_numbers.shape[0])
        if energy_window is not None:
            idx = idx[(grid.energies_ev >= energy_window[0]) & (grid.energies_ev <= energy_window[1])]
        sel = np.sort(rng.choice(idx, size=min(energies_per_case, len(idx)), replace=False))
        k, ph = grid.wave_numbers[sel], grid.phase_shifts[sel]
        feats = plan.precond_features(k, ph, F)
        N = cl.n_atoms
        atoms = rng.choice(N, size=min(atoms_per_case, N), replace=False)
        for a in atoms:
            if kind == fms.PRECOND_BLOCK:
                blk, st = plan.inverse_block(k, ph, int(a))
                ok = st == 0
                cnt = blk.shape[1]
                full = np.zeros((len(sel), Cc, Cc), np.complex128)
                full[:, :cnt, :cnt] = blk - np.eye(cnt)
                t = np.zeros((len(sel), O), np.float32)
                t[:, 0::2] = full.reshape(len(sel), -1).real
                t[:, 1::2] = full.reshape(len(sel), -1).imag
                Xs.append(feats[ok, device_index(int(a), N)])
                Ts.append(t[ok])
                continue
            diag, st = plan.inverse_diagonal(k, ph, int(a))
            ok = st == 0
            nch = diag.shape[1] // plan.inputs["nsp"]
            t = np.zeros((len(sel), O), np.float32)
            d = diag[:, ::plan.inputs["nsp"]][:, :nch] - 1.0
            t[:, 0:2 * nch:2] = d.real
            t[:, 1:2 * nch:2] = d.imag
            Xs.append(feats[ok, device_index(int(a), N)])
            Ts.append(t[ok])
        plan.close()
    return np.concatenate(Xs), np.concatenate(Ts)


def rocksalt_training_cases(n_cases: int, radius_range=(6.0, 8.0), n_energies: int = 300, seed: int = 11,
                            material_seed: int = 3):
    """Seeded rocksalt AB clusters (a = 4.44 A, sigma 0.04 A) with radii drawn from radius_range: new geometry
    (displacements, size) per case, one material -- the phase shifts of the seeded smooth model with
    `material_seed` on the energy grid -20..100 eV (the rocksalt workload uses material seed 3).  The
    preconditioner is learned for a material and carried across cluster geometries."""
    rng = np.random.default_rng(seed)
    out = []
    for c in range(n_cases):
        r = float(rng.uniform(*radius_range))
        cl = workloads.rocksalt_cluster(np.random.default_rng(seed * 1000 + c), radius=r)
        out.append((cl, workloads.energy_grid(cl, n_energies, -20.0, 100.0, seed=material_seed)))
    return out


def train_preconditioner(ctx: fms.Context, lmax: int, X, T, *, hidden: int = 64, epochs: int = 300,
                         batch_size: int = 256, learning_rate: float = 2e-3, seed: int = 0,
                         kind: int = fms.PRECOND_DIAGONAL):
    """A PrecondModel of the given kind trained on (X, T); returns (model, per-epoch full-set loss)."""
    model = fms.PrecondModel(ctx, lmax, hidden, seed, kind)
    hist = model.train(X, T, epochs=epochs, batch_size=batch_size, learning_rate=learning_rate, seed=seed)
    return model, hist
