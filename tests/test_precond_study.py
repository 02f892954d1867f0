"""What per-atom and low-rank preconditioners can give the BiCGSTAB form, on the oracle's own system matrix.

CPU study (test infrastructure: numpy BiCGSTAB on the FP64 oracle's A = I - G0 T of a seeded rocksalt cluster,
R = 5.2 A, n = 912, lmax 3), the evidence behind the learned preconditioner's form:
- the exact channel diagonal of A^-1 roughly halves the iterations just above the edge (the learned model
  predicts it);
- the exact per-atom blocks of A^-1 precondition no better than their diagonal (so the block model cannot beat
  the diagonal one);
- deflating even the exact 32 smallest eigenvalues of the diagonally preconditioned matrix on top of the
  diagonal saves under a quarter (its small eigenvalues are not isolated), so a rank-32 correction is not built;
- well above the edge neither helps.
Right preconditioning as in the product (A M y = b, x = M y), tolerance 1e-6 on |r| / |b|.
"""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).parent))
from test_oracle_properties import _intermediates  # noqa: E402

from refeff_gb300 import workloads as wl  # noqa: E402


def _bicgstab(A, b, M, tol=1e-6, maxit=4000):
    x = np.zeros_like(b)
    r = b.copy()
    rh = r.copy()
    p = np.zeros_like(b)
    v = np.zeros_like(b)
    rho = alpha = w = 1.0
    nb = np.linalg.norm(b)
    for it in range(1, maxit + 1):
        rho1 = np.vdot(rh, r)
        beta = rho1 / rho * alpha / w
        rho = rho1
        p = r + beta * (p - w * v)
        ph = M(p)
        v = A @ ph
        alpha = rho / np.vdot(rh, v)
        s = r - alpha * v
        if np.linalg.norm(s) < tol * nb:
            return it
        sh = M(s)
        t = A @ sh
        w = np.vdot(t, s) / np.vdot(t, t)
        x += alpha * ph + w * sh
        r = s - w * t
        if np.linalg.norm(r) < tol * nb:
            return it
    return maxit


def _iterations(energy_ev, columns=(0, 10)):
    held = wl.rocksalt_cluster(np.random.default_rng(99), radius=5.2)
    grid = wl.energy_grid(held, 120, -20.0, 100.0, seed=3)
    e = int(np.argmin(np.abs(grid.energies_ev - energy_ev)))
    g0, _, A = _intermediates(held, grid.wave_numbers[e], grid.phase_shifts[e])
    n, c = A.shape[0], 16
    inv = np.linalg.inv(A)
    d = np.diag(inv).copy()
    blocks = [inv[i * c:(i + 1) * c, i * c:(i + 1) * c] for i in range(n // c)]
    lam, V = np.linalg.eig(A * d[None, :])
    Z = V[:, np.argsort(np.abs(lam))[:32]]
    Ei = np.linalg.inv(Z.conj().T @ (A @ (d[:, None] * Z)))

    def deflated(x):
        q = Z @ (Ei @ (Z.conj().T @ x))
        return d * (x - A @ (d * q) + q)

    precs = {"none": lambda x: x, "diag": lambda x: d * x,
             "block": lambda x: np.concatenate([blk @ x[i * c:(i + 1) * c] for i, blk in enumerate(blocks)]),
             "diag+deflation32": deflated}
    return {k: sum(_bicgstab(A, g0[:, j].copy(), M) for j in columns) for k, M in precs.items()}


def test_per_atom_and_low_rank_preconditioners_near_the_edge():
    its = _iterations(-7.9)
    print("iterations at -7.9 eV:", its)
    assert its["diag"] < its["none"] / 1.5
    assert its["block"] >= its["diag"]
    assert its["diag+deflation32"] > 0.75 * its["diag"]


def test_nothing_helps_well_above_the_edge():
    its = _iterations(20.3)
    print("iterations at +20.3 eV:", its)
    assert its["diag"] > 0.9 * its["none"]
    assert its["block"] > 0.9 * its["none"]
