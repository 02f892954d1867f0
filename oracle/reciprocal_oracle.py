"""TEST INFRASTRUCTURE ONLY: CPU restatement of the reciprocal-space FMS integration of one energy, the checker
of refeff_fms_reciprocal_integrate / refeff_fms_reciprocal_core_hole; never shipped or called by the product.

  FmsReciprocalPlan::new / solve_k_point     crates/refeff-core/src/fms/reciprocal.rs:80-134
  FmsReciprocalAccumulator push / finish     crates/refeff-core/src/fms/reciprocal.rs:148-222
  fms_reciprocal_apply_core_hole             crates/refeff-core/src/fms/reciprocal.rs:236-302

FP64 (numpy) arithmetic; the dense solves use the oracle's own LU (oracle/fms_oracle.cpp through pyoracle).
Pinned to the reference's known answers in tests/test_reciprocal.py (crates/refeff-core/src/fms/tests/reciprocal.rs).
"""
from __future__ import annotations

import numpy as np

from . import pyoracle


def kkr_system(structure_factor, t_matrix):
    """I - G(k) T with T applied column by column over its non-zero entries, rows ascending."""
    G = np.asarray(structure_factor, dtype=np.complex128)
    T = np.asarray(t_matrix, dtype=np.complex128)
    n = G.shape[0]
    A = np.eye(n, dtype=np.complex128)
    for c in range(n):
        for inner in np.nonzero(T[:, c])[0]:
            A[:, c] -= G[:, inner] * T[inner, c]
    return A


def solve_k_point(structure_factor, t_matrix):
    A = kkr_system(structure_factor, t_matrix)
    _, X, _ = pyoracle.lu_factor_solve(A, np.asarray(structure_factor, dtype=np.complex128), mode=pyoracle.F64)
    return X


def integrate(structure_factors, weights, t_matrix):
    """sum_k w_k X_k / sum_k w_k over the k-points in mesh order."""
    weights = [float(w) for w in weights]
    if not weights:
        raise ValueError("reciprocal FMS requires at least one k-point")
    if any(not np.isfinite(w) or w <= 0.0 for w in weights):
        raise ValueError("reciprocal FMS k-point weight must be positive and finite")
    acc = None
    for G, w in zip(structure_factors, weights):
        X = solve_k_point(G, t_matrix)
        acc = X * w if acc is None else acc + X * w
    return acc / sum(weights)


def core_hole(green, absorber_offset, t_difference):
    """G - G[:, a] (I + C G_aa)^-1 C G[a, :]."""
    G = np.asarray(green, dtype=np.complex128)
    C = np.asarray(t_difference, dtype=np.complex128)
    b, a = C.shape[0], int(absorber_offset)
    if b == 0 or a + b > G.shape[0]:
        raise ValueError("absorber block outside the Green matrix")
    local = G[a:a + b, a:a + b]
    dyson = np.eye(b, dtype=np.complex128) + C @ local
    _, eff, _ = pyoracle.lu_factor_solve(dyson, C, mode=pyoracle.F64)
    return G - (G[:, a:a + b] @ eff) @ G[a:a + b, :]
