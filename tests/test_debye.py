"""Pair sigma^2 table under the correlated (idwopt 0) and classical (idwopt 3) Debye models.

The oracle is pinned to the reference's known answers (crates/refeff-core/src/debye/tests/models.rs:83-170,
crates/refeff-core/src/atomic/tests/tables_nuclear.rs:6-17) at the reference's own tolerance (1e-18 absolute);
the GPU table (refeff_fms_debye_sigma2_table) is checked against the oracle: the FP64 Debye term to 1e-13
relative (sin / exp on the GPU round differently in the last place) and the f32 table to one unit in the last
place.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from refeff_gb300 import fms, workloads as wl

KAT_TOL = 1.0e-18


# crates/refeff-core/src/debye/tests/models.rs:83-98
CORRELATION_KATS = [
    ((0.0, 400.0, 300.0, 29, 29, 2.7), False, 4.501_999_849_393_054e-3),
    ((2.55, 400.0, 300.0, 29, 29, 2.7), False, 1.691_640_883_386_128e-3),
    ((1.91, 650.0, 120.0, 29, 8, 2.3), False, 7.447_746_368_694_431e-4),
    ((0.0, 400.0, 300.0, 29, 29, 2.7), True, 4.293_628_582_101_32e-3),
    ((2.55, 400.0, 300.0, 29, 29, 2.7), True, 1.685_437_153_407_153e-3),
    ((1.91, 650.0, 120.0, 29, 8, 2.3), True, 6.129_399_740_209_465e-4),
]

# crates/refeff-core/src/debye/tests/models.rs:117-169
COPPER_PATH = [[0.0, 0.0, 0.0], [2.55, 0.0, 0.0], [0.0, 0.0, 0.0]]
TRIANGLE_PATH = [[0.0, 0.0, 0.0], [1.91, 0.25, 0.10], [2.60, 1.40, -0.20], [0.0, 0.0, 0.0]]
WALLER_KATS = [
    ((300.0, 400.0, 2.7), COPPER_PATH, [29, 29, 29], False, 5.620_717_932_013_852e-3),
    ((300.0, 400.0, 2.7), COPPER_PATH, [29, 29, 29], True, 5.216_382_857_388_334e-3),
    ((180.0, 650.0, 2.3), TRIANGLE_PATH, [29, 8, 29, 29], False, 2.623_124_881_997_499_5e-3),
    ((180.0, 650.0, 2.3), TRIANGLE_PATH, [29, 8, 29, 29], True, 1.796_449_763_322_294e-3),
]

# crates/refeff-core/src/atomic/tests/tables_nuclear.rs:6-17
WEIGHT_KATS = [(1, 1.007_899_999_618_530_3), (2, 4.002_600_193_023_682), (26, 55.849_998_474_121_094),
               (75, 186.199_996_948_242_2), (92, 238.029_998_779_296_88), (118, 294.0), (121, 330.0), (139, 392.0)]


@pytest.mark.parametrize("args,classical,want", CORRELATION_KATS)
def test_oracle_debye_correlation_kat(args, classical, want):
    got, _ = po.debye_correlation(*args, classical=classical)
    assert abs(got - want) < KAT_TOL


@pytest.mark.parametrize("temps,path,z,classical,want", WALLER_KATS)
def test_oracle_debye_waller_kat(temps, path, z, classical, want):
    assert abs(po.debye_waller(*temps, path, z, classical=classical) - want) < KAT_TOL


def test_oracle_atomic_weight_kat():
    for z, w in WEIGHT_KATS:
        assert po.atomic_weight(z) == w
    assert po.atomic_weight(0) < 0 and po.atomic_weight(140) < 0


def test_oracle_debye_rejects_invalid_inputs():
    """models.rs:101-115 and :172-190: negative rij or tk, atomic number 0, a one-row path, a Z count mismatch."""
    for args in [(-1.0, 400.0, 300.0, 29, 29, 2.7), (1.0, 400.0, -1.0, 29, 29, 2.7), (1.0, 400.0, 300.0, 29, 0, 2.7),
                 (1.0, 0.0, 300.0, 29, 29, 2.7), (1.0, 400.0, 300.0, 29, 29, 0.0)]:
        with pytest.raises(po.OracleError):
            po.debye_correlation(*args)
    with pytest.raises(po.OracleError):
        po.debye_waller(300.0, 400.0, 2.7, [[0.0, 0.0, 0.0]], [29])
    with pytest.raises(po.OracleError):  # zero-length leg
        po.debye_waller(300.0, 400.0, 2.7, [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]], [29, 29, 29])


def test_oracle_pair_table_structure():
    """fms.rs:4383-4431: zero diagonal; idwopt < 0 puts sig2g on every other entry; a Debye entry equals sigms on
    the path (atom1, atom2, atom1) plus sig2g, narrowed to f32, stored at [atom2, atom1]."""
    cl = wl.config0()[0]
    pos, pots = np.asarray(cl.positions, np.float32)[:12], np.asarray(cl.potentials)[:12]
    t, _ = po.debye_sigma2_table(-1, pos, pots, [29, 29], tk=300.0, thetad=315.0, rsavg=1.2, sig2g=0.003)
    assert (np.diag(t) == 0).all() and (t[~np.eye(12, dtype=bool)] == np.float32(0.003)).all()
    for idwopt in (0, 3):
        t, term = po.debye_sigma2_table(idwopt, pos, pots, [29, 8], tk=300.0, thetad=315.0, rsavg=1.2, sig2g=0.001)
        assert (np.diag(t) == 0).all() and (t[~np.eye(12, dtype=bool)] > 0.001).all()
        a1, a2 = 0, 5
        path = np.array([pos[a1], pos[a2], pos[a1]], np.float64)
        z = [[29, 8][pots[a1]], [29, 8][pots[a2]], [29, 8][pots[a1]]]
        s = po.debye_waller(300.0, 315.0, 1.2, path, z, classical=idwopt == 3)
        assert term[a2, a1] == s
        assert t[a2, a1] == np.float32(np.float64(np.float32(0.001)) + s)


def test_library_exports_debye_table():
    lib = fms.load()
    assert hasattr(lib, "refeff_fms_debye_sigma2_table")


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def _ulp_diff(a, b):
    ai = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    bi = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(ai - bi)


@pytest.fixture(scope="module")
def ctx():
    return fms.Context(0)


@pytest.mark.gpu
@pytest.mark.parametrize("idwopt", [0, 3])
@pytest.mark.parametrize("config", ["config0", "config1"])
def test_gpu_debye_table_matches_oracle(ctx, idwopt, config):
    cl = getattr(wl, config)()[0]
    z = [29, 8] if idwopt == 0 else [26, 47]
    kw = dict(tk=300.0, thetad=315.0, sig2g=0.0015)
    gpu, gterm = fms.debye_sigma2_table(ctx, idwopt, cl.positions, cl.potentials, z, temperature=kw["tk"],
                                        debye_temperature=kw["thetad"], average_norman_radius=1.3,
                                        sig2g=kw["sig2g"], with_debye_term=True)
    ref, rterm = po.debye_sigma2_table(idwopt, cl.positions, cl.potentials, z, rsavg=1.3, **kw)
    off = ~np.eye(len(cl.potentials), dtype=bool)
    assert np.abs(gterm - rterm)[off].max() <= 1e-13 * np.abs(rterm[off]).max()
    assert _ulp_diff(gpu, ref).max() <= 1
    assert (np.diag(gpu) == 0).all()


@pytest.mark.gpu
def test_gpu_debye_table_idwopt_negative_and_errors(ctx):
    cl = wl.config0()[0]
    pos, pots = np.asarray(cl.positions)[:10], np.asarray(cl.potentials)[:10]
    t = fms.debye_sigma2_table(ctx, -1, pos, pots, [29, 29], temperature=0.0, debye_temperature=0.0,
                               average_norman_radius=0.0, sig2g=0.004)
    assert (np.diag(t) == 0).all() and (t[~np.eye(10, dtype=bool)] == np.float32(0.004)).all()
    bad = [
        dict(idwopt=1, z=[29, 29], tk=300.0, th=315.0, rs=1.2, code=13),     # spring model: not built
        dict(idwopt=0, z=[29, 0], tk=300.0, th=315.0, rs=1.2, code=1),       # atomic number 0
        dict(idwopt=0, z=[29, 140], tk=300.0, th=315.0, rs=1.2, code=1),     # outside the weight table
        dict(idwopt=0, z=[29, 29], tk=-1.0, th=315.0, rs=1.2, code=1),       # negative tk
        dict(idwopt=3, z=[29, 29], tk=300.0, th=0.0, rs=1.2, code=1),        # thetad 0
        dict(idwopt=0, z=[29, 29], tk=300.0, th=315.0, rs=0.0, code=1),      # rnrmav 0
    ]
    for b in bad:
        with pytest.raises(fms.FmsError) as e:
            fms.debye_sigma2_table(ctx, b["idwopt"], pos, pots, b["z"], temperature=b["tk"],
                                   debye_temperature=b["th"], average_norman_radius=b["rs"])
        assert e.value.code == b["code"], b
    dup = np.array(pos, np.float32)
    dup[3] = dup[2]
    with pytest.raises(fms.FmsError) as e:   # zero-length path leg
        fms.debye_sigma2_table(ctx, 0, dup, pots, [29, 29], temperature=300.0, debye_temperature=315.0,
                               average_norman_radius=1.2)
    assert e.value.code == 1


@pytest.mark.gpu
def test_gpu_plan_with_debye_table_matches_oracle(ctx):
    """The GPU table drives the plan: gg equals the FP64 oracle fed the oracle's table (config 0, 6 energies)."""
    cl, grid = wl.config0()
    sel = np.arange(0, 100, 17)
    z = [29, 8]
    table = fms.debye_sigma2_table(ctx, 0, cl.positions, cl.potentials, z, temperature=300.0,
                                   debye_temperature=315.0, average_norman_radius=1.2)
    ref_table, _ = po.debye_sigma2_table(0, cl.positions, cl.potentials, z, tk=300.0, thetad=315.0, rsavg=1.2)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph, mean_square_displacements=table)
    got, st = fms.fms_real_space_spectrum(plan, grid.wave_numbers[sel], grid.phase_shifts[sel], fms.FORM_FP64_LU)
    assert (st == 0).all()
    want = po.fms_spectrum(cl.positions, cl.potentials, cl.lmaxph, grid.wave_numbers[sel], grid.phase_shifts[sel],
                           sigsqr=ref_table, mode=po.F64, threads=po.threads_available())
    m = plan.shape.absorber_block
    for e in range(len(sel)):
        g, w = got[e, :m, :m, 0], want[e, :m, :m, 0]
        assert np.linalg.norm(g - w) <= 1e-10 * np.linalg.norm(w)
