"""Pin the CPU oracle to the reference's known-answer tests (no GPU).

Each test mirrors one reference #[test] (cited in tests/golden/reference_kat.json)
and checks the oracle's f32-faithful mode at the reference tolerance
(2e-4 absolute for Complex32, crates/refeff-core/src/fms/tests.rs:235-240),
and the FP64 mode at the same tolerance (the KAT values are f32 results).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as po

KAT = json.loads((Path(__file__).parent / "golden" / "reference_kat.json").read_text())
TOL = KAT["tolerance"]["complex32_abs"]
MODES = [po.F32, po.F64]


def cval(entry):
    re_, im_ = entry["value"]
    return complex(re_, im_)


def assert_c(actual, entry, tol=TOL):
    expected = cval(entry)
    assert abs(complex(actual) - expected) < tol, f"{actual} vs {expected} ({entry['src']})"


def f32(x):
    return float(np.float32(x))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("case", ["xclmz_lx3", "xclmz_limited_m"])
def test_xclmz(mode, case):
    k = KAT[case]
    a = k["args"]
    t = po.polynomials(a["lx"], a["lmaxp1"], a["mmaxp1"], complex(*a["rho"]), mode)
    for key, e in k["entries"].items():
        il, im = map(int, key.split(","))
        assert_c(t[il, im], e)
    assert_c(t.sum(), k["sum"])
    assert int(np.sum(np.abs(t.real) + np.abs(t.imag) > 1e-6)) == k["nonzero"]["value"]


@pytest.mark.parametrize("mode", MODES)
def test_xclmz_rejects_invalid(mode):
    with pytest.raises(po.OracleError):
        po.polynomials(3, 0, 1, 1.0, mode)
    with pytest.raises(po.OracleError):
        po.polynomials(3, 5, 1, 1.0, mode)
    with pytest.raises(po.OracleError):
        po.polynomials(3, 1, 1, 0.0, mode)
    with pytest.raises(po.OracleError):
        po.polynomials(3, 1, 1, complex(float("nan"), 0.0), mode)


@pytest.mark.parametrize("mode", MODES)
def test_rotxan(mode):
    k = KAT["rotxan"]
    a = k["args"]
    fwd = po.rotation_matrix(a["lmax"], a["mmax"], a["beta"], a["phi"], True, mode)
    bwd = po.rotation_matrix(a["lmax"], a["mmax"], a["beta"], a["phi"], False, mode)
    assert fwd.shape == (7, 7, 4)
    assert_c(fwd.sum(), k["forward_sum"])
    assert_c(bwd.sum(), k["backward_sum"])
    nz = lambda t: int(np.sum(np.abs(t.real) + np.abs(t.imag) > 1e-6))
    assert nz(fwd) == k["forward_nonzero"]["value"]
    assert nz(bwd) == k["backward_nonzero"]["value"]
    for table, entries in ((fwd, k["forward"]), (bwd, k["backward"])):
        for key, e in entries.items():
            m2, m1, l = map(int, key.split(","))
            assert_c(table[m2 + 3, m1 + 3, l], e)


def _xgllm(mode, lx, mu, l1, l2, clm):
    out = np.zeros(2)
    buf = po.cbuf(clm)
    rc = po.lib().oracle_xgllm(mode, lx, mu, l1, l2, po.ptr(buf), po.ptr(out))
    po.check(rc)
    return complex(out[0], out[1])


@pytest.mark.parametrize("mode", MODES)
def test_xgllm(mode):
    k = KAT["xgllm"]
    clm = po.polynomials(3, 4, 4, complex(*k["args"]["rho"]), mode)
    for case in k["cases"]:
        assert_c(_xgllm(mode, 3, case["mu"], case["l1"], case["l2"], clm), case)
    with pytest.raises(po.OracleError):
        _xgllm(mode, 3, 3, 2, 3, clm)  # mu > l1 (xgllm.rs:75-80)


def _pair_tables(mode, lmax, k, positions):
    """fms_pair_tables restated on top of the oracle's polynomial kernel (pairs.rs:9-51)."""
    dt = np.float32 if mode == po.F32 else np.float64
    pos = np.asarray(positions, dtype=np.float32).astype(dt)
    n = len(pos)
    rho = np.zeros((n, n), dtype=np.complex128)
    poly = np.zeros((lmax + 1, lmax + 1, n, n), dtype=np.complex128)
    kk = np.complex64(k) if mode == po.F32 else np.complex128(k)
    for i in range(n):
        for j in range(i + 1):
            d = pos[i] - pos[j]
            dist = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
            r = complex(dt(kk.real) * dist, dt(kk.imag) * dist)
            rho[i, j] = rho[j, i] = r
            if i == j:
                continue
            clm = po.polynomials(lmax, lmax + 1, lmax + 1, r, mode)
            for l in range(lmax + 1):
                for m in range(lmax + 1):
                    poly[m, l, j, i] = poly[m, l, i, j] = clm[l, m]
    return rho, poly


@pytest.mark.parametrize("mode", MODES)
def test_pair_tables(mode):
    k = KAT["pair_tables"]
    a = k["args"]
    rho, poly = _pair_tables(mode, a["lmax"], complex(*a["k"]), a["positions"])
    for key, e in k["rho"].items():
        i, j = map(int, key.split(","))
        assert_c(rho[i, j], e)
    assert_c(poly.sum(), k["poly_sum"])
    assert int(np.sum(np.abs(poly.real) + np.abs(poly.imag) > 1e-6)) == k["poly_nonzero"]["value"]
    for key, e in k["poly"].items():
        idx = tuple(map(int, key.split(",")))
        assert_c(poly[idx], e)


def _g0_element(mode, first, second, rho, k, msd, clm, back, fwd, lx=2, L=2):
    out = np.zeros(2)
    f = np.asarray(first, dtype=np.int32)
    s = np.asarray(second, dtype=np.int32)
    rb, kb = po.cbuf([rho]), po.cbuf([k])
    cb, bb, fb = po.cbuf(clm), po.cbuf(back), po.cbuf(fwd)
    rc = po.lib().oracle_free_propagator_element(mode, lx, L, po.ptr(f), po.ptr(s), po.ptr(rb), po.ptr(kb),
                                                 float(msd), po.ptr(cb), po.ptr(bb), po.ptr(fb), po.ptr(out))
    po.check(rc)
    return complex(out[0], out[1])


@pytest.mark.parametrize("mode", MODES)
def test_free_propagator_element(mode):
    k = complex(1.2, 0.3)
    rho, _ = _pair_tables(mode, 2, k, [[0, 0, 0], [1, 2, 2]])
    clm = po.polynomials(2, 3, 3, rho[0, 1], mode)
    back = po.rotation_matrix(2, 2, 0.7, 1.1, False, mode)
    fwd = po.rotation_matrix(2, 2, 0.7, 1.1, True, mode)
    v = _g0_element(mode, [0, 2, 1, 1], [1, 2, -1, 1], rho[0, 1], k, 0.05, clm, back, fwd)
    assert_c(v, KAT["free_propagator"]["value"])
    # excluded pairs (pairs.rs:185-238): same atom / spin mismatch are zero
    assert _g0_element(mode, [0, 1, 0, 1], [0, 1, 0, 1], 0.0, k, 0.05, clm, back, fwd) == 0
    assert _g0_element(mode, [0, 1, 0, 1], [1, 1, 0, 2], rho[0, 1], k, 0.05, clm, back, fwd) == 0
    # invalid scalars (pairs.rs:240-300)
    with pytest.raises(po.OracleError):
        _g0_element(mode, [0, 1, 0, 1], [1, 1, 0, 1], rho[0, 1], k, float("inf"), clm, back, fwd)
    with pytest.raises(po.OracleError):
        _g0_element(mode, [0, 1, 0, 1], [1, 1, 0, 1], 0.0, k, 0.05, clm, back, fwd)
    with pytest.raises(po.OracleError):
        _g0_element(mode, [0, 1, 0, 1], [1, 1, 0, 1], rho[0, 1], complex(float("nan"), 0), 0.05, clm, back, fwd)


@pytest.mark.parametrize("mode", MODES)
def test_damping_uses_angstrom_units(mode):
    def pref(rho, k, msd):
        out = np.zeros(2)
        rb, kb = po.cbuf([rho]), po.cbuf([k])
        po.check(po.lib().oracle_prefactor(mode, po.ptr(rb), po.ptr(kb), float(msd), po.ptr(out)))
        return complex(out[0], out[1])
    ratio = pref(1.5, 2.0, 0.05) / pref(1.5, 2.0, 0.0)
    assert abs(ratio.real - np.exp(-0.2)) < KAT["tolerance"]["f32_abs"]
    assert abs(ratio.imag) < KAT["tolerance"]["f32_abs"]
    assert abs(pref(1.5, 0.0, 10.0) - pref(1.5, 0.0, 0.0)) < TOL


@pytest.mark.parametrize("mode", MODES)
def test_getang(mode):
    k = KAT["getang"]
    pos = np.asarray(k["positions"], dtype=np.float32)
    for case in k["cases"]:
        th, ph = np.zeros(1), np.zeros(1)
        po.lib().oracle_pair_polar_angles(mode, po.ptr(pos[case["i"]]), po.ptr(pos[case["j"]]), 0,
                                          po.ptr(th), po.ptr(ph))
        assert abs(th[0] - case["theta"]["value"]) < KAT["tolerance"]["f32_abs"]
        assert abs(ph[0] - case["phi"]["value"]) < KAT["tolerance"]["f32_abs"]
    th, ph = np.ones(1), np.ones(1)
    po.lib().oracle_pair_polar_angles(mode, po.ptr(pos[0]), po.ptr(pos[0]), 1, po.ptr(th), po.ptr(ph))
    assert th[0] == 0 and ph[0] == 0


def test_athep_sort():
    k = KAT["athep"]
    pos = np.asarray(k["positions"], dtype=np.float32).copy()
    pots = np.asarray(k["potentials"], dtype=np.int32).copy()
    keys = np.zeros(len(pots))
    po.check(po.lib().oracle_sort_atoms_by_radius(len(pots), po.ptr(pos), po.ptr(pots), po.ptr(keys)))
    assert pots.tolist() == k["sorted_potentials"]["value"]
    assert pos[0].tolist() == [0, 0, 0] and pos[1].tolist() == [-1, 0, 0]
    for got, e in zip(keys, k["keys"]):
        assert abs(got - e["value"]) < KAT["tolerance"]["f64_abs"]
    bad = np.array([[np.nan, 0, 0]], dtype=np.float32)
    assert po.lib().oracle_sort_atoms_by_radius(1, po.ptr(bad), po.ptr(np.zeros(1, np.int32)),
                                               po.ptr(np.zeros(1))) != 0


def test_sortat():
    k = KAT["sortat"]
    pos = np.asarray(k["positions"], dtype=np.float32).copy()
    pots = np.asarray(k["potentials"], dtype=np.int32).copy()
    rep = np.zeros(4, dtype=np.int64)
    po.check(po.lib().oracle_sort_representative_atoms(0, 3, len(pots), po.ptr(pos), po.ptr(pots), po.ptr(rep)))
    assert rep.tolist() == k["representatives"]["value"]
    assert pots.tolist() == k["sorted_potentials"]["value"]
    assert pos[1].tolist() == k["position_1"]["value"]
    assert pos[2].tolist() == k["position_2"]["value"]
    assert pos[3].tolist() == k["position_3"]["value"]
    # central mismatch / potential out of range (cluster.rs:225-240)
    one = np.zeros((1, 3), dtype=np.float32)
    assert po.lib().oracle_sort_representative_atoms(0, 1, 1, po.ptr(one), po.ptr(np.ones(1, np.int32)),
                                                    po.ptr(np.zeros(2, np.int64))) != 0
    assert po.lib().oracle_sort_representative_atoms(-1, 1, 1, po.ptr(one), po.ptr(np.ones(1, np.int32)),
                                                    po.ptr(np.zeros(2, np.int64))) != 0


def test_yprep_cluster():
    k = KAT["yprep"]
    pos = np.asarray(k["positions"], dtype=np.float32)
    pots = np.asarray(k["potentials"], dtype=np.int32)
    out_pos = np.zeros_like(pos)
    out_pots = np.zeros_like(pots)
    n, ca, un = (np.zeros(1, np.int32) for _ in range(3))
    po.check(po.lib().oracle_yprep_cluster(0, len(pots), po.ptr(pots), po.ptr(pos), float(k["radius"]),
                                           k["capacity"], po.ptr(out_pos), po.ptr(out_pots), po.ptr(n),
                                           po.ptr(ca), po.ptr(un)))
    assert ca[0] == k["central_atom"]["value"]
    assert un[0] == k["untruncated"]["value"]
    assert out_pots[: n[0]].tolist() == k["potentials_out"]["value"]
    assert out_pos[: n[0]].tolist() == k["positions_out"]["value"]
    dup = np.array([0, 0], np.int32)
    two = np.array([[0, 0, 0], [1, 0, 0]], np.float32)
    assert po.lib().oracle_yprep_cluster(0, 2, po.ptr(dup), po.ptr(two), 1.0, 2, po.ptr(out_pos), po.ptr(out_pots),
                                         po.ptr(n), po.ptr(ca), po.ptr(un)) != 0
    missing = np.array([0, 1], np.int32)
    assert po.lib().oracle_yprep_cluster(2, 2, po.ptr(missing), po.ptr(two), 1.0, 2, po.ptr(out_pos),
                                         po.ptr(out_pots), po.ptr(n), po.ptr(ca), po.ptr(un)) != 0


def _phases():
    ph = np.zeros((2, 5, 2), dtype=np.complex128)
    for key, v in KAT["t_matrix"]["phases"].items():
        s, l, p = map(int, key.split(","))
        ph[s, l, p] = complex(f32(v[0]), f32(v[1]))
    return ph


def _t_element(mode, nsp, first, second, pot=1, ispin=0):
    out = np.zeros(2)
    xb = po.cbuf(_phases())
    f = np.asarray(first, dtype=np.int32)
    s = np.asarray(second, dtype=np.int32)
    po.check(po.lib().oracle_t_matrix_element(mode, nsp, ispin, 2, 2, po.ptr(xb), po.ptr(f), po.ptr(s), pot,
                                              po.ptr(out)))
    return complex(out[0], out[1])


@pytest.mark.parametrize("mode", MODES)
def test_t_matrix_branches(mode):
    k = KAT["t_matrix"]
    first = [0, 2, 1, 1]
    assert_c(_t_element(mode, 1, first, first), k["non_spin"])
    assert_c(_t_element(mode, 2, first, first), k["spin_orbit_diagonal"])
    assert_c(_t_element(mode, 2, first, [0, 2, 0, 2]), k["spin_mixing"])
    assert _t_element(mode, 2, first, [1, 2, 1, 1]) == 0
    assert _t_element(mode, 2, first, [0, 2, -1, 2]) == 0


def gglu_inputs(n):
    """reference_gglu_inputs (crates/refeff-core/src/fms/tests.rs:71-90), f32-rounded."""
    g0 = np.zeros((n, n), dtype=np.complex128)
    t = np.zeros((2, n), dtype=np.complex128)
    one = np.float32
    for c in range(n):
        cf = one(c + 1)
        for r in range(n):
            rf = one(r + 1)
            if r != c:
                g0[r, c] = complex(one(0.01) * rf - one(0.02) * cf, one(0.015) * rf + one(0.005) * cf)
        t[0, c] = complex(one(0.02) * cf, one(-0.01) * cf)
        t[1, c] = complex(one(-0.005) * cf, one(0.003) * cf)
    return g0, t


def kets(nsp, atom_pots, pot_lmax, L):
    out = []
    for a, p in enumerate(atom_pots):
        for l in range(min(L, pot_lmax[p]) + 1):
            for m in range(-l, l + 1):
                for s in range(1, nsp + 1):
                    out.append([a, l, m, s])
    return np.asarray(out, dtype=np.int32)


@pytest.mark.parametrize("mode", MODES)
def test_gglu_scattering(mode):
    k = KAT["gglu"]
    ks = kets(2, [0], [1], 1)
    g0, t = gglu_inputs(len(ks))
    n = len(ks)
    sysm = np.zeros(2 * n * n)
    scat = np.zeros(2 * 8 * 8 * 1)
    po.check(po.lib().oracle_lu_scattering_explicit(
        mode, n, po.ptr(ks), 2, 1, 1, po.ptr(np.array([1], np.int32)), po.ptr(np.array([0], np.int64)), 0, 0,
        po.ptr(po.cbuf(g0)), po.ptr(po.cbuf(t)), po.ptr(sysm), po.ptr(scat)))
    A = po.from_cbuf(sysm, (n, n))
    S = po.from_cbuf(scat, (8, 8, 1))
    assert_c(A.sum(), k["system_sum"])
    assert_c(S.sum(), k["scattering_sum"])
    for key, e in k["scattering"].items():
        assert_c(S[tuple(map(int, key.split(",")))], e)
    # missing representative (solvers.rs:476-496)
    assert po.lib().oracle_lu_scattering_explicit(
        mode, n, po.ptr(ks), 2, 1, 1, po.ptr(np.array([1], np.int32)), po.ptr(np.array([-1], np.int64)), 0, 0,
        po.ptr(po.cbuf(g0)), po.ptr(po.cbuf(t)), po.ptr(sysm), po.ptr(scat)) != 0


@pytest.mark.parametrize("mode", MODES)
def test_iterative_system_matrix(mode):
    k = KAT["iterative_system"]
    ks = kets(2, [0], [1], 1)
    g0, t = gglu_inputs(len(ks))
    n = len(ks)
    for toler, sum_key, ent_key in ((0.0, "sum", "entries"), (k["cutoff_toler2"], "cutoff_sum", "cutoff_entries")):
        out = np.zeros(2 * n * n)
        po.check(po.lib().oracle_iterative_system_explicit(mode, n, po.ptr(ks), 2, po.ptr(po.cbuf(g0)),
                                                           po.ptr(po.cbuf(t)), float(toler), po.ptr(out)))
        A = po.from_cbuf(out, (n, n))
        assert_c(A.sum(), k[sum_key])
        for key, e in k[ent_key].items():
            assert_c(A[tuple(map(int, key.split(",")))], e)


@pytest.mark.parametrize("mode", MODES)
def test_cgetrf_known_answer(mode):
    k = KAT["cgetrf"]
    A = np.array([[complex(*v) for v in row] for row in k["matrix"]])
    B = np.array([[complex(*v) for v in row] for row in k["rhs"]])
    lu, x, piv = po.lu_factor_solve(A, B, mode)
    assert (piv + 1).tolist() == k["pivots_one_based"]["value"]
    F = np.array([[complex(*v) for v in row] for row in k["factors"]["value"]])
    X = np.array([[complex(*v) for v in row] for row in k["solution"]["value"]])
    assert np.max(np.abs(lu - F)) < TOL
    assert np.max(np.abs(x - X)) < TOL


def test_lu_singular_pivot_reported():
    A = np.array([[1, 2], [2, 4]], dtype=np.complex128)
    with pytest.raises(po.OracleError) as ei:
        po.lu_factor_solve(A, np.eye(2), po.F64)
    assert ei.value.code == -7


def test_driver_setup():
    k = KAT["driver_setup"]
    pots = np.asarray(k["potentials"], np.int32)
    raw = np.asarray(k["raw_lmax"], np.int32)
    plm = np.zeros(3, np.int32)
    rng = np.zeros(2, np.int32)
    rep = np.zeros(3, np.int64)
    ns = np.zeros(1, np.int32)
    k4 = np.zeros(4 * 64, np.int32)
    po.check(po.lib().oracle_driver_setup(3, po.ptr(pots), 1, 0, 2, 2, po.ptr(raw), po.ptr(plm), po.ptr(rng),
                                          po.ptr(rep), po.ptr(ns), po.ptr(k4), 64))
    assert plm.tolist() == k["potential_lmax"]["value"]
    assert rng.tolist() == k["range"]["value"]
    assert rep.tolist() == k["representative_offsets"]["value"]
    assert ns[0] == k["state_count"]["value"]
    assert k4[:4].tolist() == [0, 0, 0, 1] and k4[36:40].tolist() == [1, 0, 0, 1]
    # lfms=1 with a missing representative potential (driver.rs:62-83)
    assert po.lib().oracle_driver_setup(2, po.ptr(np.array([0, 2], np.int32)), 1, 1, 2, 1,
                                        po.ptr(np.array([1, 1, 1], np.int32)), po.ptr(plm), po.ptr(rng),
                                        po.ptr(rep), po.ptr(ns), po.ptr(k4), 64) != 0


def test_state_kets_order():
    """state.rs:158-250 known answers for the ket order."""
    pots = np.array([0, 1], np.int32)
    plm = np.zeros(2, np.int32)
    rng = np.zeros(2, np.int32)
    rep = np.zeros(2, np.int64)
    ns = np.zeros(1, np.int32)
    k4 = np.zeros(4 * 16, np.int32)
    po.check(po.lib().oracle_driver_setup(2, po.ptr(pots), 1, 1, 1, 1, po.ptr(np.array([0, 1], np.int32)),
                                          po.ptr(plm), po.ptr(rng), po.ptr(rep), po.ptr(ns), po.ptr(k4), 16))
    assert ns[0] == 5
    assert k4[:20].reshape(5, 4).tolist() == [[0, 0, 0, 1], [1, 0, 0, 1], [1, 1, -1, 1], [1, 1, 0, 1], [1, 1, 1, 1]]
    assert rep.tolist() == [0, 1]
    po.check(po.lib().oracle_driver_setup(1, po.ptr(np.array([0], np.int32)), 2, 0, 0, 1,
                                          po.ptr(np.array([1], np.int32)), po.ptr(plm), po.ptr(rng), po.ptr(rep),
                                          po.ptr(ns), po.ptr(k4), 16))
    assert ns[0] == 8
    assert k4[:16].reshape(4, 4)[:, 3].tolist() == [1, 2, 1, 2]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("minv,key", [(1, "ggbi"), (2, "ggrm"), (3, "gggm"), (4, "ggtf")])
def test_iterative_scattering_forms(mode, minv, key):
    """ggbi / ggrm / gggm / ggtf on reference_gglu_inputs(8), toler1 1e-5, toler2 0 (solvers.rs:73-292)."""
    k = KAT[key]
    ks = kets(2, [0], [1], 1)
    g0, t = gglu_inputs(len(ks))
    n = len(ks)
    sysm = np.zeros(2 * n * n)
    scat = np.zeros(2 * 8 * 8 * 1)
    order = np.zeros(1, np.int32)
    po.check(po.lib().oracle_iterative_scattering_explicit(
        mode, minv, n, po.ptr(ks), 2, 1, 1, po.ptr(np.array([1], np.int32)), po.ptr(np.array([0], np.int64)), 0, 0,
        po.ptr(po.cbuf(g0)), po.ptr(po.cbuf(t)), 1.0e-5, 0.0, po.ptr(sysm), po.ptr(scat), po.ptr(order)))
    A = po.from_cbuf(sysm, (n, n))
    S = po.from_cbuf(scat, (8, 8, 1))
    assert int(order[0]) == k["order"]["value"]
    assert_c(A.sum(), k["system_sum"])
    assert_c(S.sum(), k["scattering_sum"])
    for key_, e in k["scattering"].items():
        assert_c(S[tuple(map(int, key_.split(",")))], e)
