"""TEST INFRASTRUCTURE ONLY -- CPU restatement (numpy, float64) of the learned
preconditioner's network and features, the checker for the GPU training and
inference kernels of refeff_gb300/csrc/precond_mlp.cu.  It has no reference
counterpart: the reference's BiCGSTAB (crates/refeff-core/src/fms/internals/
iterative.rs:181-254) is unpreconditioned.

Network: X (S x F) -> tanh(X W1^T + b1) -> tanh(. W2^T + b2) -> . W3^T + b3,
parameters packed as W1[H][F], b1[H], W2[H][H], b2[H], W3[O][H], b3[O]; loss
= mean over all S x O entries of (y - t)^2.
"""
from __future__ import annotations

import numpy as np

SHELL_EDGES = (0.0, 2.9, 3.7, 4.6)


def feature_count(L: int) -> int:
    return 2 + 2 * (L + 1) + 3 * (2 + 2 * (L + 1))


def output_count(L: int, kind: int = 0) -> int:
    """Diagonal model (kind 0): Re/Im per channel; block model (kind 1): Re/Im of the C x C block, C = (L+1)^2."""
    c = (L + 1) ** 2
    return 2 * c * c if kind == 1 else 2 * c


def block_preconditioner(Y, atom_lmax, L, on):
    """The per-atom blocks the BiCGSTAB form applies for a block model's outputs Y (S x N x 2C^2, row-major,
    Re/Im interleaved): identity plus the prediction on the atom's own (lmax_atom+1)^2 channels when `on`
    (the energy lies in the model's window), the identity alone otherwise; zero beyond those channels."""
    c = (L + 1) ** 2
    Y = np.asarray(Y, np.float64)
    S, N = Y.shape[0], Y.shape[1]
    B = np.zeros((S, N, c, c), np.complex128)
    for s in range(S):
        for d in range(N):
            cnt = (int(atom_lmax[d]) + 1) ** 2
            blk = np.eye(cnt, dtype=np.complex128)
            if on[s]:
                y = Y[s, d, 0::2] + 1j * Y[s, d, 1::2]
                blk = blk + y.reshape(c, c)[:cnt, :cnt]
            B[s, d, :cnt, :cnt] = blk
    return B


def unpack(p, F, H, O):
    p = np.asarray(p, np.float64)
    i = 0
    out = []
    for shape in [(H, F), (H,), (H, H), (H,), (O, H), (O,)]:
        n = int(np.prod(shape))
        out.append(p[i:i + n].reshape(shape))
        i += n
    assert i == p.size
    return out


def forward(p, F, H, O, X):
    W1, b1, W2, b2, W3, b3 = unpack(p, F, H, O)
    X = np.asarray(X, np.float64)
    h1 = np.tanh(X @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h1, h2, h2 @ W3.T + b3


def loss_grad(p, F, H, O, X, T):
    """Loss and its analytic gradient (backpropagation), both float64."""
    W1, b1, W2, b2, W3, b3 = unpack(p, F, H, O)
    X = np.asarray(X, np.float64)
    h1, h2, y = forward(p, F, H, O, X)
    d = y - np.asarray(T, np.float64)
    loss = float(np.mean(d * d))
    dy = 2.0 * d / d.size
    gW3, gb3 = dy.T @ h2, dy.sum(0)
    d2 = (dy @ W3) * (1.0 - h2 * h2)
    gW2, gb2 = d2.T @ h1, d2.sum(0)
    d1 = (d2 @ W2) * (1.0 - h1 * h1)
    gW1, gb1 = d1.T @ X, d1.sum(0)
    return loss, np.concatenate([g.reshape(-1) for g in (gW1, gb1, gW2, gb2, gW3, gb3)])


def t_of_phase(delta):
    """t = (exp(2 i delta) - 1) / (2 i)."""
    return (np.exp(2j * np.asarray(delta)) - 1.0) / 2j


def shell_tables(pos, pot, npot):
    """Per atom and shell (< 2.9, < 3.7, < 4.6 Angstrom): (count / 12, mean distance / 5) and the
    neighbour fraction per potential."""
    pos = np.asarray(pos, np.float64)
    N = len(pot)
    info = np.zeros((N, 3, 2))
    frac = np.zeros((N, 3, npot))
    for d in range(N):
        r = np.linalg.norm(pos - pos[d], axis=1)
        for j in range(3):
            sel = (r >= SHELL_EDGES[j]) & (r < SHELL_EDGES[j + 1])
            sel[d] = False
            c = int(sel.sum())
            info[d, j, 0] = c / 12.0
            info[d, j, 1] = r[sel].mean() / 5.0 if c else 0.0
            for q in np.asarray(pot)[sel]:
                frac[d, j, q] += 1.0 / c
    return info, frac


def features(k, xphase, pos_dev, pot_dev, L, npot):
    """Features of every (energy, atom) in the given atom order: (E, N, F).  k (E, nsp) complex;
    xphase (E, nsp, 2L+1, npot) complex (spin 0 and the +l slot are used)."""
    k = np.asarray(k).reshape(len(k), -1)
    xphase = np.asarray(xphase)
    info, frac = shell_tables(pos_dev, pot_dev, npot)
    E, N = k.shape[0], len(pot_dev)
    out = np.zeros((E, N, feature_count(L)))
    for e in range(E):
        t = t_of_phase(xphase[e, 0, L:2 * L + 1, :])  # (L+1, npot)
        for d in range(N):
            f = [k[e, 0].real, k[e, 0].imag]
            for l in range(L + 1):
                f += [t[l, pot_dev[d]].real, t[l, pot_dev[d]].imag]
            for j in range(3):
                f += [info[d, j, 0], info[d, j, 1]]
                for l in range(L + 1):
                    m = np.sum(frac[d, j] * t[l])
                    f += [m.real, m.imag]
            out[e, d] = f
    return out
