"""CPU-only checks of the C ABI library: it loads, exports every declared entry
point, and its host-side cluster preparation matches the reference's known
answers (FEFF yprep + sortat).  No GPU call is made here."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as po
from refeff_gb300 import fms, workloads as wl

KAT = json.loads((Path(__file__).parent / "golden" / "reference_kat.json").read_text())


def test_library_exports_every_declared_symbol():
    lib = fms.load()
    names = fms.header_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name
    assert lib.refeff_fms_abi_version() == 1


def test_yprep_cluster_known_answer():
    k = KAT["yprep"]
    pos = np.asarray(k["positions"], np.float32)
    pots = np.asarray(k["potentials"], np.int32)
    out_pos, out_pot = fms.fms_yprep_cluster(pos, pots, max_potential=2, cluster_radius=k["radius"],
                                             cluster_capacity=k["capacity"])
    # sortat on top of yprep: the representative of potential 1 moves into the prefix
    opos = np.zeros_like(pos)
    opot = np.zeros_like(pots)
    n, ca, un = (np.zeros(1, np.int32) for _ in range(3))
    po.check(po.lib().oracle_yprep_cluster(0, len(pots), po.ptr(pots), po.ptr(pos), float(k["radius"]), k["capacity"],
                                           po.ptr(opos), po.ptr(opot), po.ptr(n), po.ptr(ca), po.ptr(un)))
    assert opot[: n[0]].tolist() == k["potentials_out"]["value"]
    rep = np.zeros(3, np.int64)
    opos2, opot2 = opos[: n[0]].copy(), opot[: n[0]].copy()
    po.check(po.lib().oracle_sort_representative_atoms(0, 2, int(n[0]), po.ptr(opos2), po.ptr(opot2), po.ptr(rep)))
    assert out_pot.tolist() == opot2.tolist()
    assert np.array_equal(out_pos, opos2)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_yprep_matches_oracle_on_shuffled_clusters(seed):
    rng = np.random.default_rng(seed)
    cl = wl.rocksalt_cluster(rng, radius=6.0)
    perm = rng.permutation(cl.n_atoms)
    shift = np.array([1.25, -0.5, 2.0], np.float32)
    pos = cl.positions[perm] + shift
    pots = cl.potentials[perm]
    out_pos, out_pot = fms.fms_yprep_cluster(pos, pots, max_potential=2, cluster_radius=5.0)
    opos = np.zeros_like(pos)
    opot = np.zeros_like(pots)
    n, ca, un = (np.zeros(1, np.int32) for _ in range(3))
    po.check(po.lib().oracle_yprep_cluster(0, len(pots), po.ptr(pots), po.ptr(pos), 5.0, len(pots), po.ptr(opos),
                                           po.ptr(opot), po.ptr(n), po.ptr(ca), po.ptr(un)))
    rep = np.zeros(3, np.int64)
    opos, opot = opos[: n[0]].copy(), opot[: n[0]].copy()
    po.check(po.lib().oracle_sort_representative_atoms(0, 2, int(n[0]), po.ptr(opos), po.ptr(opot), po.ptr(rep)))
    assert np.array_equal(out_pot, opot)
    assert np.array_equal(out_pos, opos)
    assert out_pot[0] == 0 and np.all(out_pos[0] == 0)


def test_yprep_rejects_like_the_reference():
    two = np.array([[0, 0, 0], [1, 0, 0]], np.float32)
    with pytest.raises(fms.FmsError) as e:
        fms.fms_yprep_cluster(two, [0, 0], cluster_radius=1.0)
    assert e.value.name == "DuplicateAbsorber"
    with pytest.raises(fms.FmsError) as e:
        fms.fms_yprep_cluster(two, [1, 1], cluster_radius=1.0)
    assert e.value.name == "MissingCentralAtom"
    with pytest.raises(fms.FmsError) as e:
        fms.fms_yprep_cluster(two, [0, 1], cluster_radius=-1.0)
    assert e.value.name == "InvalidClusterRadius"
    bad = two.copy()
    bad[1, 2] = np.nan
    with pytest.raises(fms.FmsError) as e:
        fms.fms_yprep_cluster(bad, [0, 1], cluster_radius=1.0)
    assert e.value.name == "NonFiniteCoordinate"


def test_named_workload_shapes():
    cl0, g0 = wl.config0()
    assert cl0.n_atoms == 43 and cl0.n_states == 688
    assert g0.wave_numbers.shape == (100, 1) and g0.phase_shifts.shape == (100, 1, 7, 2)
    cl1, g1 = wl.config1()
    assert cl1.n_atoms == 141 and cl1.n_states == 2256 and g1.wave_numbers.shape == (200, 1)
    re = g1.phase_shifts.real
    im = g1.phase_shifts.imag
    assert re.min() >= -np.pi and re.max() <= np.pi and im.min() >= 0 and im.max() <= 0.2 + 1e-7
    # the reference narrows k and the phases to Complex32
    assert np.array_equal(g1.wave_numbers, g1.wave_numbers.astype(np.complex64).astype(np.complex128))
