"""FF2X XANES mu(E) from the MKGTR trace (host code, no GPU).

The oracle restatement (oracle/ff2x_oracle.py) is pinned to the reference's lorenz / astep known answers
(crates/refeff-core/src/xscorr.rs:121-157) and to its constant-cross-section xscorr case
(crates/refeff-engine/src/ff2x/tests.rs:1127-1149, fixture 5167-5195); the product's refeff_ff2x_xanes_mu is
checked against the oracle on those cases and on seeded XANES-like inputs, for both ispec and with a vrcorr
shift.  mu is linear in the trace: the last test checks that too.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import ff2x_oracle as fo
from refeff_gb300 import fms

KAT = json.loads((Path(__file__).parent / "golden" / "reference_kat.json").read_text())


def test_oracle_lorenz_astep_known_answers():
    for case in KAT["xscorr_lorenz"]:
        got = fo.lorenz(*case["args"]["value"])
        want = complex(*case["want"]["value"])
        assert abs(got - want) <= 1e-12 * max(abs(want), 1.0)
    for case in KAT["xscorr_astep"]:
        assert abs(fo.astep(*case["args"]["value"]) - case["want"]["value"]) <= 1e-14


def test_lorentz_convolution_known_answers():
    """FEFF conv1 / conv on the reference fixture (crates/refeff-core/src/convolution/tests.rs:11-94), oracle and
    product, at the reference's 1e-12."""
    k = KAT["lorentz_conv"]
    omega = k["omega"]["value"]
    spec = [complex(*v["value"]) for v in k["spectrum"]]
    tol = k["tolerance"]["value"]
    i1, i2, x0, width = k["conv1_args"]["value"]
    assert abs(fo.conv1(omega[i1], omega[i2], spec[i1], spec[i2], x0, width) - complex(*k["conv1"]["value"])) < tol
    want = [complex(*v["value"]) for v in k["conv"]]
    for got in (fo.conv(omega, spec, 0.2), fms.ff2x_lorentz_convolve(omega, spec, 0.2)):
        assert max(abs(g - w) for g, w in zip(got, want)) < tol


def _constant_fixture():
    """ff2x/tests.rs:5167-5195: three horizontal rows at Im 0.1, a contour (1.0, 0.02), (1.0, 0.05), (1.0, 0)."""
    energy = [0.9 + 0.1j, 1.0 + 0.1j, 1.1 + 0.1j, 1.0 + 0.02j, 1.0 + 0.05j, 1.0 + 0.0j]
    return dict(energy=energy, ne1=3, fermi=1, xsec=[10j] * 6, bg=[1.0] * 6)


def test_oracle_constant_cross_section_xscorr():
    """ff2x/tests.rs:1127-1149: with a constant atomic cross section 10i and no trace, xscorr is the step:
    Im(xsec + cchi) = 10 astep(E - E_F) and cchi = i 10 (astep - 1)."""
    f = _constant_fixture()
    cchi = fo.xscorr(1, f["energy"], f["ne1"], f["fermi"], f["xsec"], f["bg"], [0j] * 6)
    for row, e in enumerate([0.9, 1.0, 1.1]):
        step = 0.5 + math.atan((e - 1.0) / 0.1) / math.pi
        assert abs((10j + cchi[row]).imag - 10.0 * step) <= 1e-12
        assert abs(cchi[row] - complex(0.0, 10.0 * (step - 1.0))) <= 1e-12


def test_product_constant_cross_section_case():
    f = _constant_fixture()
    mu, mu0, chi = fms.ff2x_xanes_mu(energy=f["energy"], ne1=3, fermi_index=1, omega=[0.9, 1.0, 1.1],
                                     cross_section=f["xsec"], background=f["bg"], trace=np.zeros(6), absolu=1)
    for row, e in enumerate([0.9, 1.0, 1.1]):
        step = 0.5 + math.atan((e - 1.0) / 0.1) / math.pi
        assert abs(mu0[row] - 10.0 * step) <= 1e-12 and abs(chi[row]) <= 1e-12 and mu[row] == mu0[row] + chi[row]


def xanes_inputs(rng, ne1=60, n_contour=8, ispec=1):
    """Seeded XANES-like rows in Hartree: a horizontal grid at Im = xloss across the Fermi level, then a
    vertical contour at Re = E_F ending at Im 0; a smooth atomic cross section with an edge step, a smooth
    background and a trace with oscillations."""
    xloss = 0.1 / fo.HARTREE_EV
    ef = 0.3
    main = np.linspace(ef - 15.0 / fo.HARTREE_EV, ef + 60.0 / fo.HARTREE_EV, ne1)
    fermi = int(np.argmin(np.abs(main - ef)))
    main[fermi] = ef
    contour = ef + 1j * np.r_[np.linspace(0.2, 0.9, n_contour - 1) * xloss, 0.0]
    energy = np.r_[main + 1j * xloss, contour]
    ne = energy.shape[0]
    x = energy.real - ef
    xsec = 1j * (2.0 + 0.5 * np.tanh(40.0 * x)) + 0.05 * rng.normal(size=ne)
    bg = 1.0 + 0.3 * np.exp(-3.0 * np.abs(x)) + 0.01 * rng.normal(size=ne)
    trace = (0.2 * np.exp(1j * (9.0 * x + rng.uniform(0, 6)))) * (1 + 0.1 * rng.normal(size=ne))
    omega = main + 8.979  # photon energies (Hartree), a Cu K edge offset
    return dict(energy=energy, ne1=ne1, fermi=fermi, omega=omega, xsec=xsec, bg=bg, trace=trace,
                fermi_photon=omega[fermi])


@pytest.mark.parametrize("ispec,vrcorr,include_atomic,absolu,vicorr",
                         [(1, 0.0, True, 0, 0.0), (2, 0.0, True, 0, 0.0), (1, 0.5 / 27.211396, True, 0, 0.0),
                          (1, 0.0, False, 1, 0.0), (-2, -0.4 / 27.211396, True, 0, 0.0),
                          (1, 0.0, True, 0, 1.5 / 27.211396), (2, 0.3 / 27.211396, True, 0, 0.8 / 27.211396),
                          (1, 0.0, False, 0, 0.8 / 27.211396)])
def test_product_matches_oracle(ispec, vrcorr, include_atomic, absolu, vicorr):
    rng = np.random.default_rng(7 + ispec)
    d = xanes_inputs(rng)
    got = fms.ff2x_xanes_mu(energy=d["energy"], ne1=d["ne1"], fermi_index=d["fermi"], omega=d["omega"],
                            cross_section=d["xsec"], background=d["bg"], trace=d["trace"], s02=0.9, ispec=ispec,
                            absolu=absolu, include_atomic=include_atomic, real_correction=vrcorr,
                            imaginary_correction=vicorr, fermi_photon_energy=d["fermi_photon"])
    want = fo.xanes_mu(energy=list(d["energy"]), ne1=d["ne1"], fermi=d["fermi"], omega=list(d["omega"]),
                       cross_section=list(d["xsec"]), background=list(d["bg"]), trace=list(d["trace"]), s02=0.9,
                       ispec=ispec, absolu=absolu, include_atomic=include_atomic, vrcorr=vrcorr, vicorr=vicorr,
                       fermi_photon_energy=d["fermi_photon"])
    for g, w in zip(got, want):
        w = np.asarray(w)
        assert np.abs(g - w).max() <= 1e-12 * max(np.abs(w).max(), 1.0)


def test_vrcorr_without_atomic_background_is_rejected():
    """With the atomic background off, the atomic xscorr sees a zero Fermi-level xmu, which a vrcorr shift
    cannot rescale: the reference bails there (ff2x.rs:4526-4529), and so do both restatements."""
    d = xanes_inputs(np.random.default_rng(9))
    with pytest.raises(fms.FmsError):
        fms.ff2x_xanes_mu(energy=d["energy"], ne1=d["ne1"], fermi_index=d["fermi"], omega=d["omega"],
                          cross_section=d["xsec"], background=d["bg"], trace=d["trace"], include_atomic=False,
                          real_correction=0.3 / 27.211396, fermi_photon_energy=d["fermi_photon"])
    with pytest.raises(ZeroDivisionError):
        fo.xanes_mu(energy=list(d["energy"]), ne1=d["ne1"], fermi=d["fermi"], omega=list(d["omega"]),
                    cross_section=list(d["xsec"]), background=list(d["bg"]), trace=list(d["trace"]),
                    include_atomic=False, vrcorr=0.3 / 27.211396, fermi_photon_energy=d["fermi_photon"])


def test_mu_is_affine_in_the_trace():
    """mu(trace) - mu(0) is linear: doubling the trace doubles chi, and mu0 does not depend on the trace."""
    d = xanes_inputs(np.random.default_rng(3))
    kw = dict(energy=d["energy"], ne1=d["ne1"], fermi_index=d["fermi"], omega=d["omega"], cross_section=d["xsec"],
              background=d["bg"], fermi_photon_energy=d["fermi_photon"])
    _, m0a, ca = fms.ff2x_xanes_mu(trace=d["trace"], **kw)
    _, m0b, cb = fms.ff2x_xanes_mu(trace=2.0 * d["trace"], **kw)
    assert np.abs(m0a - m0b).max() == 0.0
    assert np.abs(cb - 2.0 * ca).max() <= 1e-12 * np.abs(ca).max()


def test_invalid_rows_are_rejected():
    d = xanes_inputs(np.random.default_rng(5))
    kw = dict(energy=d["energy"], fermi_index=d["fermi"], omega=d["omega"], cross_section=d["xsec"],
              background=d["bg"], trace=d["trace"])
    with pytest.raises(fms.FmsError):
        fms.ff2x_xanes_mu(ne1=len(d["energy"]), **kw)          # no contour rows
    bad = dict(kw)
    bad["trace"] = d["trace"].copy()
    bad["trace"][4] = np.nan
    with pytest.raises(fms.FmsError) as e:
        fms.ff2x_xanes_mu(ne1=d["ne1"], **bad)
    assert e.value.code == 6


@pytest.mark.parametrize("sig_gk", [0.0, 5e-5, 0.02, 0.08])
def test_debye_factor_matches_oracle(sig_gk):
    """FF2X's sig_gk Debye factor (ff2x.rs:3388-3397): chi damped by exp(-(sig_gk k)^2) above the 1e-4
    threshold, mu = mu0 + chi, through the C ABI against the oracle."""
    rng = np.random.default_rng(4)
    k = np.linspace(0.0, 12.0, 57)
    mu0 = 1.0 + 0.1 * rng.normal(size=57)
    chi = 0.05 * rng.normal(size=57)
    mu, c = fms.ff2x_debye_factor(k, sig_gk, mu0, chi)
    mu_o, c_o = fo.debye_factor(k, sig_gk, mu0, chi)
    assert np.allclose(c, c_o, rtol=1e-15, atol=0) and np.allclose(mu, mu_o, rtol=1e-15, atol=1e-17)
    if sig_gk <= 1e-4:
        assert np.array_equal(c, chi)
    else:
        assert abs(c[-1]) < abs(chi[-1])


# ---------------------------------------------------------------------------
# thermal xscorr (electronic temperature > 0)
# ---------------------------------------------------------------------------

def _thermal_fixture():
    """ff2x/tests.rs:5197-5238 through the audited known-answer file: 17 xsect.dat rows (3 horizontal at Im 0.2,
    3 loss rows at Im 0.1, 10 auxiliary / pole rows, the Fermi row (1.0, 0)), cross section 10i, background 1."""
    k = KAT["thermal_xscorr"]
    energy = [complex(*v["value"]) for v in k["energy"]]
    ne = len(energy)
    return dict(energy=energy, ne1=k["ne1"]["value"], xsec=[complex(*k["cross_section"]["value"])] * ne,
                bg=[k["background"]["value"]] * ne, temp=k["temperature_ev"]["value"],
                want=k["corrected_im"]["value"], tol=k["tolerance"]["value"])


def test_oracle_thermal_xscorr_known_answer():
    """tests.rs:1152-1178: at 0.5 eV the thermal xscorr of the constant cross section gives Im(xsec + cchi) =
    2.5858..., 5.0000..., 7.4141... on the three horizontal rows, and cchi = i (those - 10)."""
    f = _thermal_fixture()
    ne = len(f["energy"])
    cchi = fo.thermal_xscorr(1, f["energy"], f["ne1"], f["xsec"], f["bg"], [0j] * ne, 0.0, f["temp"])
    for row, want in enumerate(f["want"]):
        assert abs(cchi[row] - complex(0.0, want - 10.0)) <= f["tol"]
        assert abs((f["xsec"][row] + cchi[row]).imag - want) <= f["tol"]


def test_product_thermal_xscorr_known_answer():
    f = _thermal_fixture()
    ne = len(f["energy"])
    cchi = fms.ff2x_xscorr(energy=f["energy"], ne1=f["ne1"], fermi_index=1, cross_section=f["xsec"],
                           background=f["bg"], path_chi=np.zeros(ne), electronic_temperature=f["temp"])
    for row, want in enumerate(f["want"]):
        assert abs(cchi[row] - complex(0.0, want - 10.0)) <= f["tol"]
    # through the XANES step: mu0 = the corrected atomic cross section, no fine structure
    mu, mu0, chi = fms.ff2x_xanes_mu(energy=f["energy"], ne1=f["ne1"], fermi_index=1, omega=[0.9, 1.0, 1.1],
                                     cross_section=f["xsec"], background=f["bg"], trace=np.zeros(ne), absolu=1,
                                     electronic_temperature=f["temp"])
    assert np.abs(mu0 - np.array(f["want"])).max() <= f["tol"] and np.abs(chi).max() <= 1e-12


@pytest.mark.parametrize("ispec,vrcorr,temp", [(1, 0.0, 0.5), (2, 0.0, 0.3), (1, 0.01, 0.4), (1, 0.0, 1.0)])
def test_product_thermal_xscorr_matches_oracle(ispec, vrcorr, temp):
    """A non-constant xmu (seeded cross section and trace on a 7-point horizontal grid): the product's C++ and
    the oracle's restatement agree (the contour, residue and Fermi-Lorentz terms all non-trivial)."""
    rng = np.random.default_rng(int(temp * 10) + ispec)
    ne1 = 7
    hor = [complex(0.7 + 0.1 * i, 0.15) for i in range(ne1)]
    loss = [complex(0.7 + 0.1 * i, 0.08) for i in range(ne1)]
    aux = [complex(1.0, 0.01 * (i + 1)) for i in range(10)]
    poles = [complex(1.0 + 0.003 * i, 0.02 * (i + 1)) for i in range(4)]
    energy = hor + loss + aux + poles + [complex(1.0, 0.0)]
    ne = len(energy)
    xsec = list(rng.normal(size=ne) * 0.3 + 1j * (8.0 + rng.normal(size=ne)))
    bg = list(1.0 + 0.1 * rng.random(ne))
    chia = list(rng.normal(size=ne) * 0.2 + 1j * rng.normal(size=ne) * 0.2)
    want = fo.thermal_xscorr(ispec, energy, ne1, xsec, bg, chia, vrcorr, temp)
    got = fms.ff2x_xscorr(energy=energy, ne1=ne1, fermi_index=3, cross_section=xsec, background=bg, path_chi=chia,
                          ispec=ispec, real_correction=vrcorr, electronic_temperature=temp)
    scale = max(abs(w) for w in want)
    assert max(abs(g - w) for g, w in zip(got, want)) <= 1e-10 * scale


def test_thermal_xscorr_rejects_short_layouts_and_bad_temperatures():
    f = _thermal_fixture()
    ne = len(f["energy"])
    with pytest.raises(fms.FmsError):  # 2 ne1 + 11 rows needed
        fms.ff2x_xscorr(energy=f["energy"][:12] + [1.0 + 0j], ne1=3, fermi_index=1, cross_section=f["xsec"][:13],
                        background=f["bg"][:13], path_chi=np.zeros(13), electronic_temperature=0.5)
    with pytest.raises(fms.FmsError):
        fms.ff2x_xscorr(energy=f["energy"], ne1=3, fermi_index=1, cross_section=f["xsec"], background=f["bg"],
                        path_chi=np.zeros(ne), electronic_temperature=-0.1)


# ---- xsect.dat reader and the rdxbin handoff (crates/refeff-io/src/xsect_dat.rs) ----

def _xsect_text(scalars, gamach_ev, ne1, ik0, energy, background, cross_section, title="Cu crystal"):
    """xsect.dat records in FEFF's layout (the reader takes any decimal field, so full precision is kept)."""
    out = [f"# {title}", "#  " + "-" * 71]
    out.append("# " + "".join(f" {v:.17e}" for v in scalars) + " method to calculate xsect")
    out.append(f"#  {gamach_ev:.17e} {ne1:6d} {ik0:6d} gamach in eV, # of points on horizontal axis")
    out.append("#       em              xsnorm            xsec  ")
    for e, b, x in zip(energy, background, cross_section):
        out.append(f"  {e.real:.17e} {e.imag:.17e} {b:.17e} {x.real:.17e} {x.imag:.17e}")
    return "\n".join(out) + "\n"


def _close(a, b, tol):
    return abs(a - b) <= tol * max(1.0, abs(b))


def test_xsect_dat_parses_reference_records(tmp_path):
    """The codec's comment-prefixed records parse to what the reference's parse test asserts."""
    k = KAT["xsect_dat_parse"]
    p = tmp_path / "xsect.dat"
    p.write_text(k["text"]["text"])
    d = fms.ff2x_read_xsect_dat(p, s02=0.05)
    assert d["rows"] == 2 and d["titles"] == 1
    assert d["ne1"] == k["main_energy_count"]["value"]
    assert d["fermi_index"] == k["fermi_index"]["value"] - 1
    e0 = d["energy"][0] * 27.211396
    assert _close(e0.real, k["energy_0"]["value"][0], 1e-14) and _close(e0.imag, k["energy_0"]["value"][1], 1e-14)
    assert d["cross_section"][1] == complex(*k["cross_section_1"]["value"])
    assert d["s02"] == 0.85 and d["file_s02"] == 0.85


def test_xsect_dat_ff2x_handoff_matches_reference(tmp_path):
    """Energies in Hartree, omega, signed wave numbers and the core-hole width of the reference's three-row
    handoff test, to its 1e-14 tolerance; S02 follows FEFF's rule."""
    k = KAT["xsect_ff2x_handoff"]
    energy = [complex(*v["value"]) for v in k["energy_ev"]]
    xsec = [complex(*v["value"]) for v in k["cross_section"]]
    p = tmp_path / "xsect.dat"
    p.write_text(_xsect_text(k["scalars"]["value"], k["core_hole_width_ev"]["value"], k["ne1"]["value"],
                             k["ik0"]["value"], energy, k["background"]["value"], xsec))
    s02, mbconv = k["s02_args"]["value"]
    d = fms.ff2x_read_xsect_dat(p, s02=s02, mbconv=mbconv)
    tol = k["tolerance"]["value"]
    assert d["rows"] == 3 and d["ne1"] == 2 and d["fermi_index"] == 0
    assert _close(d["core_hole_width"], k["core_hole_width_hartree"]["value"], tol)
    assert _close(d["s02"], 0.85, tol) and _close(d["edge"], 9.1, tol) and _close(d["emu"], -0.4, tol)
    for r in range(3):
        want = k["energy_hartree"][r]["value"]
        assert _close(d["energy"][r].real, want[0], tol) and _close(d["energy"][r].imag, want[1], tol), r
        assert _close(d["omega"][r], k["omega_hartree"]["value"][r], tol), r
        assert _close(d["wave_number"][r], k["wave_number"]["value"][r], tol), r
        assert d["cross_section"][r] == xsec[r] and d["background"][r] == k["background"]["value"][r]
    for case in ("s02_keep", "s02_file"):
        cur, mb = k[case]["args"]["value"]
        assert _close(fms.ff2x_read_xsect_dat(p, s02=cur, mbconv=mb)["s02"], k[case]["want"]["value"], tol)


def test_xsect_dat_feeds_the_xanes_step(tmp_path):
    """Seeded XANES rows written as an xsect.dat (energies in eV, edge 0 and emu set so that omega is the rows'
    photon energies), read back and handed to FF2X: mu(E) from the file equals mu(E) from the rows themselves,
    and both equal the oracle's."""
    d = xanes_inputs(np.random.default_rng(3))
    emu = float(d["omega"][0] - d["energy"][0].real)
    p = tmp_path / "xsect.dat"
    p.write_text(_xsect_text([0.9, 0.0, 0.0, 0.0, emu], 1.5, d["ne1"], d["fermi"] + 1,
                             d["energy"] * 27.211396, d["bg"], d["xsec"]))
    h = fms.ff2x_read_xsect_dat(p, s02=0.9)
    assert h["rows"] == d["energy"].shape[0] and h["ne1"] == d["ne1"] and h["fermi_index"] == d["fermi"]
    assert np.allclose(h["energy"], d["energy"], rtol=1e-15, atol=1e-17)
    assert np.allclose(h["omega"][:d["ne1"]], d["omega"], rtol=1e-14, atol=0)
    kw = dict(ne1=h["ne1"], fermi_index=h["fermi_index"], trace=d["trace"], s02=h["s02"],
              fermi_photon_energy=d["fermi_photon"])
    got = fms.ff2x_xanes_mu(energy=h["energy"], omega=h["omega"][:h["ne1"]], cross_section=h["cross_section"],
                            background=h["background"], **kw)
    direct = fms.ff2x_xanes_mu(energy=d["energy"], omega=d["omega"], cross_section=d["xsec"], background=d["bg"],
                               **kw)
    want = fo.xanes_mu(energy=list(h["energy"]), ne1=h["ne1"], fermi=h["fermi_index"],
                       omega=list(h["omega"][:h["ne1"]]), cross_section=list(h["cross_section"]),
                       background=list(h["background"]), trace=list(d["trace"]), s02=h["s02"],
                       fermi_photon_energy=d["fermi_photon"])
    for g, r, w in zip(got, direct, want):
        w = np.asarray(w)
        scale = max(np.abs(w).max(), 1.0)
        assert np.abs(g - r).max() <= 1e-12 * scale
        assert np.abs(g - w).max() <= 1e-12 * scale


@pytest.mark.parametrize("text,fragment", [
    ("# Cu\n# title without separator\n", "separator"),
    ("# Cu\n#  -----------------------------------------------------------------------\n# nope\n", "method"),
    ("# Cu\n#  --------\n# 1 2 3 4 5\n# 1.0 1 1\n# nothing here\n 1 2 3 4 5\n", "label"),
    ("# Cu\n#  --------\n# 1 2 3 4 5\n# 1.0 2 1\n# em xsnorm xsec\n 1 2 3 4 5\n", "ne1"),
    ("# Cu\n#  --------\n# 1 2 3 4 5\n# 1.0 1 0\n# em xsnorm xsec\n 1 2 3 4 5\n", "Fermi index"),
    ("# Cu\n#  --------\n# 1 2 3 4 5\n# 1.0 1 1\n# em xsnorm xsec\n 1 2 3 4\n", "fields"),
    ("# Cu\n#  --------\n# 1 2 3 4 5\n# 1.0 1 1\n# em xsnorm xsec\n 1 2 3 4 1.0D+00\n", "not a number"),
    ("# Cu\n#  --------\n# 1 2 3 4 5\n# 1.0 1 1\n# em xsnorm xsec\n", "at least one"),
])
def test_xsect_dat_rejects_bad_records(tmp_path, text, fragment):
    p = tmp_path / "xsect.dat"
    p.write_text(text)
    with pytest.raises(fms.FmsError) as err:
        fms.ff2x_read_xsect_dat(p)
    assert fragment in str(err.value), str(err.value)
