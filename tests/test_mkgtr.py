"""MKGTR: transition B matrix, gg trace, fms.bin / gtr.dat and the `mkgtr` stage.

Known answers:
  bcoef B matrices          crates/refeff-core/src/angular/tests.rs:284-412, 948-1007
  getgtr traces             crates/refeff-core/src/fms/tests/mkgtr.rs:4-70
  engine MKGTR consistency  crates/refeff-engine/src/fms/tests.rs:529-563 (fms.bin trace == recomputed, 2e-6)
"""
import numpy as np
import pytest

from oracle import feff_files as ff
from oracle import pyoracle
from refeff_gb300 import fms

PTZ = [[0.20 - 0.05j, -0.10 + 0.04j, 0.03 + 0.02j],
       [0.11 - 0.07j, 0.50, -0.08 + 0.09j],
       [0.06 + 0.01j, 0.13 - 0.02j, 0.17 + 0.03j]]
BASE = dict(lmax=3, initial_kappa=-1, polarization=1, polarization_tensor=PTZ, multipole=2, trace_orbital=False,
            spin=1, spin_channels=1, spin_vector_angle=0.3)
IDX = [(0, 0, 1, 0, 0, 1), (1, 0, 2, -1, 0, 2), (0, 1, 4, 0, 1, 4), (-1, 0, 5, 1, 1, 6), (0, 0, 7, 0, 0, 7),
       (0, 0, 8, 0, 0, 8)]
# (overrides, kappas, lind, six values, sum, nonzero count) -- angular/tests.rs:284-412
KATS = [
    (dict(polarization=0), [-2, 1, 0, 0, 0, -1, 2, -3], [1, 1, -1, -1, -1, 0, 2, 2],
     [-0.05555555555555555, 0, 0, 0, 0.02, 0.02], -0.06666666666666678, 34),
    ({}, [-2, 1, 0, 0, 0, -1, 2, -3], [1, 1, -1, -1, -1, 0, 2, 2],
     [-0.06273441744900005 - 0.002816883591316175j, 0, 0, 0, 0.028021517059414094 + 0.0012286136649168643j,
      0.032783586221432195 + 0.001621399287040505j], -0.1498383428670292 + 1.0054312926918387j, 776),
    (dict(trace_orbital=True), None, None,
     [-0.13927806177774438 - 0.006120603534129609j, 0, 0, 0, 0.08851128918371495 - 0.0038584833449001833j,
      0.08464910571422107 + 0.0008909740920669523j], -0.31619310063452616 + 0.8078421709741431j, 728),
    (dict(spin=0), None, None,
     [-0.12775761018690238 - 0.0018521924356471728j, 0, 0, 0, 0.05865146715590615 - 0.0005346566843031169j,
      0.06730612780091635 + 0.0012482092313231155j], -0.2170418650429801 + 1.3409109998393136j, 828),
    (dict(initial_kappa=2, multipole=1, spin=2, spin_vector_angle=-0.4), [1, -2, 3, 0, -1, 2, -3, 0],
     [1, 1, 3, -1, 0, 2, 2, -1],
     [-0.04864195024406099 + 0.003463869265078493j, 0.0017631363458188638 - 0.0002788047964405202j, 0, 0,
      0.035984450619728485 + 0.0004976156588231403j, 0], 0.21773917179567237 + 1.463795753151296j, 1432),
]


def _val(bm, m2, s2, k2, m1, s1, k1, L=3):
    return bm[m2 + L, s2, k2 - 1, m1 + L, s1, k1 - 1]


def _check_kat(bm, li, ki, kat):
    _, kap, lnd, vals, total, nnz = kat
    if kap is not None:
        assert list(ki) == kap and list(li) == lnd
    for t, v in zip(IDX, vals):
        assert abs(_val(bm, *t) - v) < 1e-12
    assert abs(bm.sum() - total) < 1e-12
    assert np.count_nonzero(np.abs(bm) > 1e-14) == nnz


@pytest.mark.parametrize("kat", KATS, ids=["averaged", "polarized", "traced", "spin_folded", "magnetic_dipole"])
def test_oracle_transition_matrix_known_answers(kat):
    kw = dict(BASE)
    kw.update(kat[0])
    _check_kat(*pyoracle.transition_b_matrix(**kw), kat)


@pytest.mark.parametrize("kat", KATS, ids=["averaged", "polarized", "traced", "spin_folded", "magnetic_dipole"])
def test_product_transition_matrix_matches_known_answers_and_oracle(kat):
    kw = dict(BASE)
    kw.update(kat[0])
    bm, li, ki = fms.transition_matrix(**kw)
    _check_kat(bm, li, ki, kat)
    ob, oli, oki = pyoracle.transition_b_matrix(**kw)
    assert np.array_equal(li, oli) and np.array_equal(ki, oki)
    assert np.abs(bm - ob).max() <= 1e-15


@pytest.mark.parametrize("lmax,kappa,mult,spin,nsp", [(1, -1, 0, 0, 1), (2, 1, 1, 1, 2), (4, -2, 2, -1, 2),
                                                     (2, -4, 2, 2, 1)])
def test_product_transition_matrix_matches_oracle_more_edges(lmax, kappa, mult, spin, nsp):
    for pol in (0, 1):
        kw = dict(lmax=lmax, initial_kappa=kappa, polarization=pol, polarization_tensor=PTZ, multipole=mult,
                  spin=spin, spin_channels=nsp, spin_vector_angle=0.7)
        bm, li, ki = fms.transition_matrix(**kw)
        ob, oli, oki = pyoracle.transition_b_matrix(**kw)
        assert np.array_equal(li, oli) and np.array_equal(ki, oki)
        assert np.abs(bm - ob).max() <= 1e-15


def _sample_bmat(lind, entries, L=0):
    ML = 2 * L + 1
    bm = np.zeros((ML, 2, 8, ML, 2, 8), complex)
    for idx, v in entries.items():
        bm[idx] = v
    return bm, np.array(lind, np.int32)


def test_oracle_trace_known_answers():
    # mkgtr.rs:4-37: two spectra, one s-channel, gg 1x1
    b1, li = _sample_bmat([0, -1, -1, -1, -1, -1, -1, -1], {(0, 0, 0, 0, 0, 0): 2.0 + 0.5j})
    b2, _ = _sample_bmat([0, -1, -1, -1, -1, -1, -1, -1], {(0, 0, 0, 0, 0, 0): -1.0 + 0.25j})
    gg = np.array([[[complex(np.float32(1.0), np.float32(2.0))]], [[complex(np.float32(-0.5), np.float32(0.75))]]])
    rkk = np.zeros((2, 8, 1), complex)
    rkk[0, 0, 0], rkk[1, 0, 0] = 3.0 - 1.0j, 0.5 + 2.0j
    tr = pyoracle.mkgtr_trace(gg, [b1, b2], [li, li], rkk, nsp=1, lmax=0)
    assert abs(tr[0, 0] - gg[0, 0, 0] * b1[0, 0, 0, 0, 0, 0] * rkk[0, 0, 0] ** 2) < 1e-12
    assert abs(tr[1, 1] - gg[1, 0, 0] * b2[0, 0, 0, 0, 0, 0] * rkk[1, 0, 0] ** 2) < 1e-12
    # mkgtr.rs:40-70: spin channel indexing (row = (l^2+l+m) nsp + s)
    b3, li3 = _sample_bmat([0, -1, -1, -1, -1, -1, -1, -1], {(0, 1, 0, 0, 0, 0): 1.5 - 0.25j})
    g2 = np.zeros((1, 2, 2), complex)
    g2[0, 0, 1] = 0.5 - 0.25j
    rk2 = np.zeros((1, 8, 2), complex)
    rk2[0, 0, 0], rk2[0, 0, 1] = 2.0, 3.0 + 0.5j
    tr2 = pyoracle.mkgtr_trace(g2, [b3], [li3], rk2, nsp=2, lmax=0)
    assert abs(tr2[0, 0] - g2[0, 0, 1] * b3[0, 1, 0, 0, 0, 0] * rk2[0, 0, 0] * rk2[0, 0, 1]) < 1e-12


def _awkward_traces(rng, nspec, ne):
    t = (rng.normal(size=(nspec, ne)) + 1j * rng.normal(size=(nspec, ne))) * 10.0 ** rng.integers(-12, 6, (nspec, ne))
    t.flat[0] = 0.0
    if t.size > 1:
        t.flat[1] = -1e-40 + 2e39j
    return t


def test_write_fms_bin_and_gtr_dat_byte_exact(tmp_path):
    rng = np.random.default_rng(2)
    for nspec, ne, npad in [(1, 1, 8), (1, 37, 8), (3, 11, 6), (2, 5, 10)]:
        tr = _awkward_traces(rng, nspec, ne)
        fms.write_fms_bin(tmp_path / "fms.bin", tr, cluster_radius=3.25, nph=2, pad_width=npad)
        assert (tmp_path / "fms.bin").read_text() == ff.fms_bin_text(tr, cluster_radius=3.25, nph=2, pad_width=npad)
        grid = rng.normal(size=ne) * 20 + 0.1j
        tr0 = np.round(tr[0], 3)
        fms.write_gtr_dat(tmp_path / "gtr.dat", grid, tr0)
        assert (tmp_path / "gtr.dat").read_text() == ff.gtr_dat_text(grid, tr0)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("nsp,lmax", [(1, 1), (2, 2), (1, 3)])
def test_gpu_trace_matches_oracle(nsp, lmax):
    ctx = fms.Context(0)
    rng = np.random.default_rng(10 * nsp + lmax)
    E, dim = 9, nsp * (lmax + 1) ** 2
    gg = rng.normal(size=(E, dim, dim)) + 1j * rng.normal(size=(E, dim, dim))
    rkk = rng.normal(size=(E, 8, nsp)) + 1j * rng.normal(size=(E, 8, nsp))
    mats = [fms.transition_matrix(lmax=lmax, initial_kappa=k, polarization=p, polarization_tensor=PTZ, multipole=2,
                                  spin=1, spin_channels=nsp, spin_vector_angle=0.2)
            for k, p in [(-1, 1), (1, 0), (-2, 1)]]
    bm, li = [m[0] for m in mats], [m[1] for m in mats]
    got = fms.mkgtr_trace(ctx, gg, bm, li, rkk, active_spin_channels=nsp, lmax=lmax)
    want = pyoracle.mkgtr_trace(gg, bm, li, rkk, nsp=nsp, lmax=lmax)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
def test_gpu_trace_fused_on_device_scattering_tables():
    torch = pytest.importorskip("torch")
    from refeff_gb300 import workloads as wl
    ctx = fms.Context(0)
    cl, grid = wl.small_cluster(2.6, lmax=2, n_energies=5, seed=3)
    plan = fms.fms_real_space_plan(ctx, cl.positions, cl.potentials, cl.lmaxph)
    scat, _ = fms.fms_real_space_spectrum(plan, grid.wave_numbers, grid.phase_shifts)
    E, Cc, npot, m = scat.shape[0], plan.shape.channel_count, plan.inputs["npot"], plan.shape.absorber_block
    d_tab = torch.from_numpy(np.ascontiguousarray(np.stack([scat[e].reshape(-1, order="F") for e in range(E)]))).cuda()
    rng = np.random.default_rng(4)
    rkk = rng.normal(size=(E, 8, 1)) + 1j * rng.normal(size=(E, 8, 1))
    d_rkk = torch.from_numpy(np.ascontiguousarray(rkk.reshape(-1, order="F"))).cuda()
    d_tr = torch.zeros(E, dtype=torch.complex128, device="cuda")
    bm, li, _ = fms.transition_matrix(lmax=2, initial_kappa=-1, polarization=0, multipole=0, spin=0)
    fms.mkgtr_trace_device(ctx, E, m, 1, 2, [bm], [li], d_tab.data_ptr(), Cc, Cc * Cc * npot, d_rkk.data_ptr(),
                           d_tr.data_ptr())
    want = pyoracle.mkgtr_trace(scat[:, :m, :m, 0], [bm], [li], rkk, nsp=1, lmax=2)[0]
    got = d_tr.cpu().numpy()
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
def test_mkgtr_stage_on_reference_fixture(tmp_path):
    ctx = fms.Context(0)
    ff.reference_engine_fixture(tmp_path)
    fms.run_fms_in_dir(ctx, tmp_path, fms.FORM_FP64_LU)
    assert not (tmp_path / "fms.bin").exists()
    assert fms.run_mkgtr_in_dir(ctx, tmp_path) == 2
    # oracle: gg.bin narrowed to complex64 (fms.rs:5883-5918), bcoef with the fixture's global.inp, rkk q=0
    gg = np.array(ff.parse_gg_dat((tmp_path / "gg.bin").read_text()))
    gg = gg.real.astype(np.float32).astype(float) + 1j * gg.imag.astype(np.float32).astype(float)
    bm, li, _ = pyoracle.transition_b_matrix(lmax=1, initial_kappa=-1, polarization=0,
                                             polarization_tensor=np.eye(3) / 3.0, multipole=0, spin=0,
                                             spin_channels=1, spin_vector_angle=0.0)
    rkk = ff.read_rkk((tmp_path / "phase.bin").read_text(), nsp=1, ne=2)
    want = pyoracle.mkgtr_trace(gg, [bm], [li], rkk, nsp=1, lmax=1)
    radius, counts, spectra = ff.parse_fms_bin((tmp_path / "fms.bin").read_text())
    assert radius == 3.0 and counts == [2, 2, 0, 1, 8, 0]
    assert spectra.shape == (1, 2)
    assert np.abs(spectra - want).max() <= 2e-6  # the engine test's bound
    assert np.abs(spectra - want).max() <= 1e-11 * np.abs(want).max()
    assert (tmp_path / "fms.bin").read_text().splitlines()[0] == "FMS rfms= 3.0000"
    pb = fms.read_phase_bin(tmp_path / "phase.bin")
    assert (tmp_path / "gtr.dat").read_text() == ff.gtr_dat_text(pb["energy_grid"], spectra[0])
    log = (tmp_path / "log3.dat").read_text()
    assert "Done with module: FMS." in log and log.endswith(
        "\nMKGTR: Tracing over Green's function ...\nDone with module: MKGTR.\n")
    # cached: nothing regenerated, the log keeps one MKGTR block
    assert fms.run_mkgtr_in_dir(ctx, tmp_path) == 0
    assert (tmp_path / "log3.dat").read_text() == log


@pytest.mark.gpu
def test_mkgtr_stage_unsupported_projections(tmp_path):
    ctx = fms.Context(0)
    ff.reference_engine_fixture(tmp_path)
    fms.run_fms_in_dir(ctx, tmp_path)
    (tmp_path / "global.inp").write_text(ff.global_inp_text(0, do_nrixs=1))
    with pytest.raises(fms.FmsError) as e:
        fms.run_mkgtr_in_dir(ctx, tmp_path)
    assert e.value.code == 13
    (tmp_path / "global.inp").write_text(ff.global_inp_text(0))
    (tmp_path / "eels.inp").write_text("ELNES\n")
    with pytest.raises(fms.FmsError) as e:
        fms.run_mkgtr_in_dir(ctx, tmp_path)
    assert e.value.code == 13
