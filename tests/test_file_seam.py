"""FEFF file seam: gg.dat / gg.bin writer, phase.bin reader and the work-directory
entry point, checked against the oracle-side restatement of the reference's
codecs (oracle/feff_files.py) and the reference's own known-answer strings.

Known answers:
  E20.10 / E13.5 fields     crates/refeff-io/src/format.rs:509-527
  gg.dat value line         crates/refeff-io/src/gg_dat.rs:687
  PAD zero                  crates/refeff-io/src/pad.rs:124-125
  source-generated gg shape crates/refeff-engine/src/fms/tests.rs:529-563
"""
import cmath
import math

import numpy as np
import pytest

from oracle import feff_files as ff
from oracle import pyoracle
from refeff_gb300 import fms


# ---------------------------------------------------------------------------
# oracle codecs pinned to the reference's known answers
# ---------------------------------------------------------------------------

def test_oracle_fortran_exp_matches_reference_known_answers():
    assert ff.fortran_exp(0.0380998403, 20, 10) == "    0.3809984030E-01"
    assert ff.fortran_exp(-4.3629, 13, 5) == " -0.43629E+01"
    assert ff.fortran_exp(0.0, 13, 5) == "  0.00000E+00"
    assert ff.fortran_exp(-0.0, 13, 5) == " -0.00000E+00"
    assert ff.fortran_exp(-0.2936442169, 20, 10, 3) == "  -0.2936442169E+000"


def test_oracle_gg_dat_matches_reference_value_line():
    text = ff.gg_dat_text([np.array([[1.0 - 2.5j]])])
    assert text.endswith("    0.1000000000E+01    -0.2500000000E+01\n")
    assert text.startswith("#SN#   Section:    1\n#DF# This section written in txt.\n#H#\n"
                           "#DT# 2D complex array with sizes    1   1\n")


def test_oracle_pad_zero_and_round_trip():
    assert ff.pad_encode(0.0, 8) == "Q%%%%%%%"
    assert ff.pad_decode("Q%%%%%%%", 8) == 0.0
    rng = np.random.default_rng(3)
    for v in list(rng.normal(size=200) * 10.0 ** rng.integers(-12, 12, size=200)) + [1.0, -1.0, 0.1, 1e-30, 7e30]:
        d = ff.pad_decode(ff.pad_encode(float(v), 8), 8)
        assert abs(d - v) <= abs(v) * 1e-11 + 1e-300  # 8 characters hold about 13 digits


# ---------------------------------------------------------------------------
# product host codecs (no GPU needed) against the oracle restatement
# ---------------------------------------------------------------------------

def _awkward_sections(rng, n, dim):
    mag = 10.0 ** rng.integers(-15, 8, size=(n, dim, dim, 2))
    v = rng.normal(size=(n, dim, dim, 2)) * mag
    v[0, 0, 0] = (0.0, -0.0)
    v[0, 0, -1] = (-0.0, 1.0)
    v[-1, -1, 0] = (9.99999999995, 0.099999999995)
    v[-1, 0, 0] = (1e-200, -5e150)
    return v[..., 0] + 1j * v[..., 1]


def test_write_gg_dat_byte_exact(tmp_path):
    rng = np.random.default_rng(11)
    for n, dim in [(1, 1), (3, 4), (2, 18)]:
        sec = _awkward_sections(rng, n, dim)
        path = tmp_path / f"gg_{n}_{dim}.dat"
        fms.write_gg_dat(path, sec)
        assert path.read_text() == ff.gg_dat_text(list(sec))


def _kat(name):
    import json
    from pathlib import Path
    kat = json.loads((Path(__file__).parent / "golden" / "reference_kat.json").read_text())[name]
    idx = {tuple(int(i) for i in key.split(",")): complex(*v["value"]) for key, v in kat["entries"].items()}
    return bytes.fromhex(kat["bytes"]["hex"]), tuple(kat["shape"]["value"]), idx


@pytest.mark.parametrize("name", ["gg_slice_bin", "gg_diag_bin"])
def test_oracle_rhorrp_codecs_match_reference_bytes(name):
    """FEFF gg_slice.bin / gg_diag.bin byte streams of the reference codec tests (rhorrp_gg_bin.rs:785-835):
    the oracle parses them to the asserted shape and values and writes them back byte for byte."""
    data, shape, entries = _kat(name)
    parse, write = ((ff.parse_gg_slice_bin, ff.gg_slice_bin_bytes) if name == "gg_slice_bin" else
                    (ff.parse_gg_diag_bin, ff.gg_diag_bin_bytes))
    v = parse(data)
    assert v.shape == shape
    for key, want in entries.items():
        assert v[key] == np.complex64(want), key
    assert write(v) == data


def test_write_rhorrp_bins_byte_exact(tmp_path):
    """The product's gg_slice.bin / gg_diag.bin writers reproduce the reference byte streams from the decoded
    values, and agree with the oracle on larger random blocks (values narrowed to complex f32)."""
    sl_bytes, _, _ = _kat("gg_slice_bin")
    dg_bytes, _, _ = _kat("gg_diag_bin")
    fms.write_gg_slice_bin(tmp_path / "s.bin", ff.parse_gg_slice_bin(sl_bytes))
    fms.write_gg_diag_bin(tmp_path / "d.bin", ff.parse_gg_diag_bin(dg_bytes))
    assert (tmp_path / "s.bin").read_bytes() == sl_bytes
    assert (tmp_path / "d.bin").read_bytes() == dg_bytes
    rng = np.random.default_rng(4)
    sl = rng.normal(size=(3, 16, 48)) + 1j * rng.normal(size=(3, 16, 48)) * 10.0 ** rng.integers(-30, 30, (3, 16, 48))
    dg = rng.normal(size=(2, 5, 9, 9)) - 1j * rng.normal(size=(2, 5, 9, 9))
    fms.write_gg_slice_bin(tmp_path / "s2.bin", sl)
    fms.write_gg_diag_bin(tmp_path / "d2.bin", dg)
    assert (tmp_path / "s2.bin").read_bytes() == ff.gg_slice_bin_bytes(sl)
    assert (tmp_path / "d2.bin").read_bytes() == ff.gg_diag_bin_bytes(dg)
    sl[1, 2, 3] = 1e39  # overflows f32: not finite after narrowing
    with pytest.raises(fms.FmsError) as e:
        fms.write_gg_slice_bin(tmp_path / "s3.bin", sl)
    assert e.value.code == 6


def test_write_gg_dat_empty_and_parse_round_trip(tmp_path):
    fms.write_gg_dat(tmp_path / "empty.dat", np.zeros((0, 4, 4), complex))
    assert (tmp_path / "empty.dat").read_text() == ""
    sec = np.array([[[1.0 - 0.5j, 2.0 + 2.5j], [3.0, -4.0 + 0.75j]]])
    fms.write_gg_dat(tmp_path / "g.dat", sec)
    back = ff.parse_gg_dat((tmp_path / "g.dat").read_text())
    assert len(back) == 1 and np.array_equal(back[0], sec[0])


def _phase_potentials(rng, ne, nsp, lmaxes):
    pots = []
    for lm in lmaxes:
        ph = rng.normal(size=(ne, 2 * lm + 1, nsp)) * 0.3 + 1j * np.abs(rng.normal(size=(ne, 2 * lm + 1, nsp))) * 0.05
        pots.append((lm, 29, "Cu", ph))
    return pots


@pytest.mark.parametrize("nsp,lmaxes,ne", [(1, [2, 2], 2), (2, [3, 1, 2], 7), (1, [0], 1)])
def test_phase_bin_read_round_trip(tmp_path, nsp, lmaxes, ne):
    rng = np.random.default_rng(5 + ne)
    grid = rng.normal(size=ne) + 1j * np.abs(rng.normal(size=ne)) * 0.1
    eref = rng.normal(size=(ne, nsp)) * 0.01 + 1j * rng.normal(size=(ne, nsp)) * 1e-3
    pots = _phase_potentials(rng, ne, nsp, lmaxes)
    (tmp_path / "phase.bin").write_text(ff.phase_bin_text(nsp=nsp, energy_grid=grid, reference_energy=eref,
                                                          potentials=pots))
    pb = fms.read_phase_bin(tmp_path / "phase.bin")

    def dec(z):
        return complex(ff.pad_decode(ff.pad_encode(z.real, 8), 8), ff.pad_decode(ff.pad_encode(z.imag, 8), 8))

    assert np.array_equal(pb["energy_grid"], np.array([dec(z) for z in grid]))
    assert np.array_equal(pb["reference_energy"], np.vectorize(dec)(eref))
    assert list(pb["potential_lmax"]) == lmaxes
    lm = max(lmaxes)
    for p, (lmp, _, _, ph) in enumerate(pots):
        got = pb["phase_shifts"][:, :, :, p]
        expect = np.zeros((ne, 2 * lm + 1, nsp), complex)
        expect[:, lm - lmp: lm + lmp + 1, :] = np.vectorize(dec)(ph)
        assert np.array_equal(got, expect)


def test_phase_bin_missing_file_is_an_error(tmp_path):
    with pytest.raises(fms.FmsError):
        fms.read_phase_bin(tmp_path / "nope.bin")


# ---------------------------------------------------------------------------
# the work-directory entry point on the GPU
# ---------------------------------------------------------------------------

BOHR = 0.529177249


def _wave_number(em, er):
    """fms_wave_numbers (crates/refeff-engine/src/fms.rs:4972-4985): sqrt(2 (E - Eref)) / bohr in f64 by the
    polar form, narrowed to complex64."""
    z = complex(2.0 * (em.real - er.real), 2.0 * (em.imag - er.imag))
    if z.imag == 0.0 or z.real == 0.0:
        w = cmath.sqrt(z)
    else:
        r, th = math.hypot(z.real, z.imag), math.atan2(z.imag, z.real)
        w = complex(math.sqrt(r) * math.cos(th / 2.0), math.sqrt(r) * math.sin(th / 2.0))
    return np.complex64(complex(w.real / BOHR, w.imag / BOHR))


def _oracle_gg(work, positions, pots, lmaxph, rdirec, sigsqr=None, sig2g=0.0):
    pb = fms.read_phase_bin(work / "phase.bin")
    ne, nsp = pb["reference_energy"].shape
    L, npot, lm = max(lmaxph), len(lmaxph), max(pb["potential_lmax"])
    k = np.array([[_wave_number(pb["energy_grid"][e], pb["reference_energy"][e, s]) for s in range(nsp)]
                  for e in range(ne)])
    xp = np.zeros((ne, nsp, 2 * L + 1, npot), complex)
    for p in range(npot):
        for sl in range(-lmaxph[p], lmaxph[p] + 1):
            xp[:, :, sl + L, p] = pb["phase_shifts"][:, sl + lm, :, p].astype(np.complex64)
    scat = pyoracle.fms_spectrum(np.asarray(positions, np.float32), pots, lmaxph, k, xp, nsp=nsp, rdirec=rdirec,
                                 sigsqr=sigsqr, sig2g=sig2g)
    m = nsp * (lmaxph[0] + 1) ** 2
    return scat[:, :m, :m, 0]


@pytest.mark.gpu
@pytest.mark.parametrize("form", [fms.FORM_FP64_LU, fms.FORM_FP32_REFINED])
def test_run_dir_reference_fixture(tmp_path, form):
    ctx = fms.Context(0)
    ff.reference_engine_fixture(tmp_path)
    rep = fms.run_fms_in_dir(ctx, tmp_path, form)
    assert rep["energies_failed"] == 0
    gg_text = (tmp_path / "gg.dat").read_text()
    assert (tmp_path / "gg.bin").read_bytes() == (tmp_path / "gg.dat").read_bytes()
    secs = ff.parse_gg_dat(gg_text)
    assert len(secs) == 2 and all(s.shape == (4, 4) for s in secs)
    assert ff.gg_dat_text(secs) == gg_text
    want = _oracle_gg(tmp_path, [[0, 0, 0], [1.4, 0, 0]], [0, 1], [1, 1], 5.0)
    got = np.array(secs)
    assert np.abs(got).max() > 1e-8
    # E20.10 keeps 10 significant digits; FP64 solves agree to 1e-10, refined ones to 1e-6
    tol = 1e-9 if form == fms.FORM_FP64_LU else 1e-6
    assert np.abs(got - want).max() <= tol * np.abs(want).max()
    log = (tmp_path / "log3.dat").read_text()
    for line in ["FMS calculation of full Green's function ...", "Using     2 energy points.",
                 "Done with module: FMS."]:
        assert line in log


@pytest.mark.gpu
def test_run_dir_larger_cluster_and_output_spin_capacity(tmp_path):
    """rocksalt-like cluster read from geom.dat (absorber not first in the file), lmaxph [2, 3], nspu 2 from
    .dimensions.dat: sections are widened with zeros (fms.rs:2004-2047)."""
    from refeff_gb300 import workloads as wl
    ctx = fms.Context(0)
    rng = np.random.default_rng(21)
    cl = wl.small_cluster(3.2, lmax=3, n_energies=1, seed=4)[0]
    pos = np.asarray(cl.positions, float)
    pots = [int(p) for p in cl.potentials]
    order = np.r_[np.arange(1, len(pots)), 0]  # absorber last in the file
    ne = 5
    grid = 0.5 + 0.4 * np.arange(ne) + 0.03j
    phase_pots = _phase_potentials(rng, ne, 1, [3] * (max(pots) + 1))
    ff.write_workdir(tmp_path, positions=pos[order], potentials=[pots[i] for i in order],
                     lmaxph=[2] + [3] * max(pots), energy_grid=grid, phase_potentials=phase_pots, rfms2=100.0,
                     rdirec=100.0, nspu=2)
    fms.run_fms_in_dir(ctx, tmp_path, fms.FORM_FP64_LU)
    secs = ff.parse_gg_dat((tmp_path / "gg.dat").read_text())
    assert len(secs) == ne and all(s.shape == (18, 18) for s in secs)
    got = np.array(secs)
    assert np.abs(got[:, 9:, :]).max() == 0 and np.abs(got[:, :, 9:]).max() == 0
    cpos, cpots = fms.fms_yprep_cluster(pos[order], [pots[i] for i in order], cluster_radius=100.0)
    want = _oracle_gg(tmp_path, cpos, cpots, [2] + [3] * max(pots), 100.0)
    assert np.abs(got[:, :9, :9] - want).max() <= 1e-9 * np.abs(want).max()


@pytest.mark.gpu
@pytest.mark.parametrize("minv", [0, 2])
def test_run_dir_save_gg_slice(tmp_path, minv):
    """save_gg_slice on: gg.bin / gg.dat as before, plus gg_slice.bin and gg_diag.bin of the full scattering
    matrix (fms.rs:1113-1125, 3659-3683), equal to the oracle's after narrowing to complex f32; minv != 0 is
    forced back to the LU form."""
    from refeff_gb300 import workloads as wl
    ctx = fms.Context(0)
    rng = np.random.default_rng(41)
    cl = wl.small_cluster(3.0, lmax=2, n_energies=1, seed=6)[0]
    pos = np.asarray(cl.positions, float)
    pots = [int(p) for p in cl.potentials]
    ne = 3
    grid = 0.7 + 0.45 * np.arange(ne) + 0.05j
    phase_pots = _phase_potentials(rng, ne, 1, [2] * (max(pots) + 1))
    lmaxph = [2] * (max(pots) + 1)
    ff.write_workdir(tmp_path, positions=pos, potentials=pots, lmaxph=lmaxph, energy_grid=grid,
                     phase_potentials=phase_pots, rfms2=100.0, rdirec=100.0)
    (tmp_path / "fms.inp").write_text(ff.fms_inp_text(lmaxph=lmaxph, rfms2=100.0, rdirec=100.0, minv=minv,
                                                      save_gg_slice=True))
    fms.run_fms_in_dir(ctx, tmp_path, fms.FORM_FP32_REFINED)
    sl = ff.parse_gg_slice_bin((tmp_path / "gg_slice.bin").read_bytes())
    dg = ff.parse_gg_diag_bin((tmp_path / "gg_diag.bin").read_bytes())
    assert ff.gg_slice_bin_bytes(sl) == (tmp_path / "gg_slice.bin").read_bytes()
    cpos, cpots = fms.fms_yprep_cluster(pos, pots, cluster_radius=100.0)
    pb = fms.read_phase_bin(tmp_path / "phase.bin")
    k = np.array([[_wave_number(pb["energy_grid"][e], pb["reference_energy"][e, 0])] for e in range(ne)])
    xp = np.zeros((ne, 1, 5, len(lmaxph)), complex)
    for p in range(len(lmaxph)):
        xp[:, :, :, p] = pb["phase_shifts"][:, :, :, p].transpose(0, 2, 1).astype(np.complex64)
    want_sl, want_dg = pyoracle.full_scattering(cpos, cpots, lmaxph, k, xp)
    n = len(cpots) * 9
    assert sl.shape == (ne, 9, n) and dg.shape == (ne, len(cpots), 9, 9)
    # complex f32 values of FP64 solves: one rounding of each part
    assert np.abs(sl - want_sl).max() <= 2e-7 * np.abs(want_sl).max()
    assert np.abs(dg - want_dg).max() <= 2e-7 * np.abs(want_dg).max()
    gg = np.array(ff.parse_gg_dat((tmp_path / "gg.dat").read_text()))
    assert np.abs(gg - want_dg[:, 0]).max() <= 1e-9 * np.abs(want_dg[:, 0]).max()


@pytest.mark.gpu
def test_run_dir_rejects_unsupported_and_inconsistent_inputs(tmp_path):
    ctx = fms.Context(0)
    ff.reference_engine_fixture(tmp_path)
    for idwopt in (1, 2, 4, 5):  # spring, sig2.dat and DMDW models are outside this library
        (tmp_path / "fms.inp").write_text(ff.fms_inp_text(lmaxph=[1, 1], rfms2=3.0, rdirec=5.0, idwopt=idwopt,
                                                          tk=300.0, thetad=315.0))
        with pytest.raises(fms.FmsError) as e:
            fms.run_fms_in_dir(ctx, tmp_path)
        assert e.value.code == 13
    (tmp_path / "fms.inp").write_text(ff.fms_inp_text(lmaxph=[1], rfms2=3.0, rdirec=5.0))
    with pytest.raises(fms.FmsError) as e:
        fms.run_fms_in_dir(ctx, tmp_path)
    assert e.value.code == 1
    (tmp_path / "fms.inp").write_text(ff.fms_inp_text(lmaxph=[3, 1], rfms2=3.0, rdirec=5.0))
    with pytest.raises(fms.FmsError) as e:
        fms.run_fms_in_dir(ctx, tmp_path)
    assert e.value.code == 5
    assert not (tmp_path / "gg.dat").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("idwopt", [0, 3])
def test_run_dir_debye_damping(tmp_path, idwopt):
    """idwopt 0 / 3: the pair sigma^2 table comes from the correlated / classical Debye model with phase.bin's
    rnrmav and atomic numbers (fms.rs:4345-4433); gg equals the oracle fed the oracle's own table, and the log
    names the model (fms.rs:6048-6058)."""
    from refeff_gb300 import workloads as wl
    ctx = fms.Context(0)
    rng = np.random.default_rng(31)
    cl = wl.small_cluster(3.2, lmax=2, n_energies=1, seed=5)[0]
    pos = np.asarray(cl.positions, float)
    pots = [int(p) for p in cl.potentials]
    ne = 4
    grid = 0.6 + 0.5 * np.arange(ne) + 0.04j
    phase_pots = _phase_potentials(rng, ne, 1, [2] * (max(pots) + 1))
    phase_pots = [(lm, z, lab, ph) for (lm, _, lab, ph), z in zip(phase_pots, [29, 8, 26, 47][:len(phase_pots)])]
    ff.write_workdir(tmp_path, positions=pos, potentials=pots, lmaxph=[2] * (max(pots) + 1), energy_grid=grid,
                     phase_potentials=phase_pots, rfms2=100.0, rdirec=100.0, sig2g=0.002, idwopt=idwopt, tk=300.0,
                     thetad=315.0)
    fms.run_fms_in_dir(ctx, tmp_path, fms.FORM_FP64_LU)
    got = np.array(ff.parse_gg_dat((tmp_path / "gg.dat").read_text()))
    cpos, cpots = fms.fms_yprep_cluster(pos, pots, cluster_radius=100.0)
    zs = [p[1] for p in phase_pots]
    table, _ = pyoracle.debye_sigma2_table(idwopt, cpos, cpots, zs, tk=300.0, thetad=315.0, rsavg=1.2, sig2g=0.002)
    assert table.max() > 0.002
    want = _oracle_gg(tmp_path, cpos, cpots, [2] * (max(pots) + 1), 100.0, sigsqr=table)
    plain = _oracle_gg(tmp_path, cpos, cpots, [2] * (max(pots) + 1), 100.0, sig2g=0.002)
    assert np.abs(want - plain).max() > 1e-6 * np.abs(want).max()   # the damping changes gg
    assert np.abs(got - want).max() <= 1e-9 * np.abs(want).max()
    model = "a Correlated Debye model" if idwopt == 0 else "the Classical Debye model"
    assert f"Applying Debye-Waller factors using {model}." in (tmp_path / "log3.dat").read_text()


@pytest.mark.gpu
def test_run_dir_cluster_from_feff_inp(tmp_path):
    """A work directory with feff.inp and no geom.dat: the stage takes its cluster from feff.inp through the
    geom.dat text FEFF's rdinp would write, so gg.dat equals the run on that geom.dat byte for byte."""
    from refeff_gb300 import workloads as wl
    ctx = fms.Context(0)
    rng = np.random.default_rng(5)
    cl = wl.small_cluster(3.2, lmax=2, n_energies=1, seed=4)[0]
    pos = np.asarray(cl.positions, float) + np.array([1.25, -0.5, 2.0])   # absorber off the origin
    pots = [int(p) for p in cl.potentials]
    order = rng.permutation(len(pots))
    lines = ["POTENTIALS"] + [f" {p} 29 Cu" for p in range(max(pots) + 1)] + ["ATOMS"]
    lines += [f" {pos[i, 0]:.6f} {pos[i, 1]:.6f} {pos[i, 2]:.6f} {pots[i]}" for i in order] + ["END"]
    ne = 3
    grid = 0.5 + 0.4 * np.arange(ne) + 0.03j
    phase_pots = _phase_potentials(rng, ne, 1, [2] * (max(pots) + 1))
    runs = {}
    for name in ("from_feff_inp", "from_geom_dat"):
        d = tmp_path / name
        ff.write_workdir(d, positions=pos, potentials=pots, lmaxph=[2] * (max(pots) + 1), energy_grid=grid,
                         phase_potentials=phase_pots, rfms2=100.0, rdirec=100.0)
        (d / "geom.dat").unlink()
        (d / "feff.inp").write_text("\n".join(lines) + "\n")
        if name == "from_geom_dat":
            fms.write_geom_dat(d / "feff.inp", d / "geom.dat")
        rep = fms.run_fms_in_dir(ctx, d, fms.FORM_FP64_LU)
        assert rep["energies_failed"] == 0
        runs[name] = (d / "gg.dat").read_bytes()
    assert runs["from_feff_inp"] == runs["from_geom_dat"]
    assert not (tmp_path / "from_feff_inp" / "geom.dat").exists()
