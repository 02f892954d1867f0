"""Reciprocal-space FMS (FEFF kkrintegral, crates/refeff-core/src/fms/reciprocal.rs): the k-point integration of
(I - G(k) T)^-1 G(k) on the GPU and the host core-hole Dyson update, against the oracle restatement
(oracle/reciprocal_oracle.py), which is pinned to the reference's identity tests
(crates/refeff-core/src/fms/tests/reciprocal.rs): the one-site resolvent average, the scalar and 2x2 Dyson
updates, and the rejected inputs.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import reciprocal_oracle as ro
from refeff_gb300 import fms

KAT = json.loads((Path(__file__).parent / "golden" / "reference_kat.json").read_text())


def _c(entry):
    return complex(*entry["value"])


def _one_site():
    k = KAT["reciprocal_one_site"]
    t = _c(k["t"])
    gs = [_c(g) for g in k["structure_factors"]]
    w = k["weights"]["value"]
    expected = sum(wi * g / (1.0 - g * t) for g, wi in zip(gs, w)) / sum(w)
    return t, gs, w, expected, k["tolerance"]["value"]


def test_oracle_one_site_resolvent_average():
    t, gs, w, expected, tol = _one_site()
    got = ro.integrate([np.array([[g]]) for g in gs], w, np.array([[t]]))
    assert abs(got[0, 0] - expected) <= 1e-14


def test_oracle_and_product_core_hole_identities():
    k = KAT["reciprocal_core_hole_scalar"]
    g, c = _c(k["green"]), _c(k["t_difference"])
    want = g / (1.0 + c * g)
    assert abs(ro.core_hole(np.array([[g]]), 0, np.array([[c]]))[0, 0] - want) <= 1e-14
    assert abs(fms.reciprocal_core_hole(np.array([[g]]), 0, np.array([[c]]))[0, 0] - want) <= 1e-14
    k = KAT["reciprocal_core_hole_2x2"]
    G = np.array([[_c(v) for v in row] for row in k["green"]])
    C = np.array([[_c(v) for v in row] for row in k["t_difference"]])
    want = np.linalg.solve(np.eye(2) + G @ C, G)   # G - G (I + C G)^-1 C G = (I + G C)^-1 G
    assert np.abs(ro.core_hole(G, 0, C) - want).max() <= 1e-14
    assert np.abs(fms.reciprocal_core_hole(G, 0, C) - want).max() <= 1e-14


def test_core_hole_on_a_larger_lattice_block_matches_oracle():
    rng = np.random.default_rng(3)
    n, b, a = 40, 9, 18
    G = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) * 0.2
    C = (rng.normal(size=(b, b)) + 1j * rng.normal(size=(b, b))) * 0.1
    assert np.abs(fms.reciprocal_core_hole(G, a, C) - ro.core_hole(G, a, C)).max() <= 1e-13


def test_rejected_inputs():
    with pytest.raises(ValueError):
        ro.integrate([np.array([[1.0]])], [0.0], np.array([[0.5]]))
    with pytest.raises(ValueError):
        ro.integrate([], [], np.array([[0.5]]))
    G = np.full((2, 2), 0.1 + 0j)
    with pytest.raises(ValueError):
        ro.core_hole(G, 2, np.array([[0.2]]))
    with pytest.raises(fms.FmsError) as e:
        fms.reciprocal_core_hole(G, 2, np.array([[0.2]]))
    assert e.value.code == 1


def _lattice_case(rng, n, K, nsp_pairs=True):
    """Seeded structure factors of moderate norm and a lattice T: diagonal per state plus, for spin pairs,
    one spin-mixing partner per row (the sparsity the reference plan assumes)."""
    G = (rng.normal(size=(K, n, n)) + 1j * rng.normal(size=(K, n, n))) * (0.6 / np.sqrt(n))
    T = np.diag(rng.normal(size=n) * 0.3 + 1j * np.abs(rng.normal(size=n)) * 0.2)
    if nsp_pairs:
        for i in range(0, n - 1, 2):
            T[i, i + 1] = 0.05 * (rng.normal() + 1j * rng.normal())
    w = rng.uniform(0.5, 2.0, size=K)
    return G, w, T


@pytest.mark.gpu
def test_gpu_one_site_known_answer():
    ctx = fms.Context(0)
    t, gs, w, expected, tol = _one_site()
    for form in (fms.FORM_FP64_LU, fms.FORM_FP32_REFINED):
        got, st = fms.reciprocal_integrate(ctx, np.array([[[g]] for g in gs]), w, np.array([[t]]), form)
        assert (st == 0).all() and abs(got[0, 0] - expected) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("n,K", [(16, 40), (50, 7), (96, 300)])
def test_gpu_integration_matches_oracle(n, K):
    """FP64 LU <= 1e-10 and the refined form <= 1e-6 (n <= 64) against the oracle; K = 300 spans batches."""
    ctx = fms.Context(0)
    G, w, T = _lattice_case(np.random.default_rng(n + K), n, K)
    want = ro.integrate(list(G), w, T)
    got, st = fms.reciprocal_integrate(ctx, G, w, T, fms.FORM_FP64_LU)
    assert (st == 0).all()
    assert np.linalg.norm(got - want) <= 1e-10 * np.linalg.norm(want)
    if n <= 64:
        got32, st32 = fms.reciprocal_integrate(ctx, G, w, T, fms.FORM_FP32_REFINED)
        assert (st32 == 0).all()
        assert np.linalg.norm(got32 - want) <= 1e-6 * np.linalg.norm(want)


@pytest.mark.gpu
def test_gpu_rejects_singular_kkr_and_bad_weights():
    """T = 1 and G(k) = 1 make I - G T singular (reciprocal.rs tests:123-131); a zero weight is rejected."""
    ctx = fms.Context(0)
    with pytest.raises(fms.FmsError) as e:
        fms.reciprocal_integrate(ctx, np.ones((1, 1, 1)), [1.0], np.ones((1, 1)))
    assert e.value.code == 9
    with pytest.raises(fms.FmsError) as e:
        fms.reciprocal_integrate(ctx, np.ones((1, 1, 1)) * 0.5, [0.0], np.ones((1, 1)) * 0.3)
    assert e.value.code == 1
