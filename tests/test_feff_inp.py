"""The cluster from feff.inp (refeff_fms_geometry_from_feff_inp / refeff_fms_write_geom_dat) through the C ABI,
against the reference's own rdinp known answers and the oracle restatement (oracle/feff_files.py).

Pinned: crates/refeff-io/src/rdinp/tests/global_geometry.rs:291-320 (the exact geom.dat of a sorted relative
cluster) and :150-185 (no potential-0 atom: the first atom is the absorber, model atoms [1, 2]).  The strict
selection sort on the fused distance (rdinp/geometry.rs:61-88) decides the order of equal-distance shells; the
oracle reproduces it with exactly rounded fused multiply-adds, and the product must give the same rows byte for
byte on fcc shells listed in shuffled order.
"""
import numpy as np
import pytest

from oracle import feff_files as ff
from refeff_gb300 import fms

REF_SORTED = """
POTENTIALS
0 29 Cu
1 29 Cu
ATOMS
0.0 0.0 0.0 0 Cu0
2.0 0.0 0.0 1 Cu2
1.0 0.0 0.0 1 Cu1
END
"""

REF_SORTED_GEOM = (
    "nat, nph =     3    1\n"
    "    1    2\n"
    " iat     x       y        z       iph  \n"
    " -----------------------------------------------------------------------\n"
    "   1      0.00000      0.00000      0.00000   0   1\n"
    "   2      1.00000      0.00000      0.00000   1   1\n"
    "   3      2.00000      0.00000      0.00000   1   1\n"
)


def _write(tmp_path, text, name="feff.inp"):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_reference_sorted_relative_cluster_geom_dat(tmp_path):
    inp = _write(tmp_path, REF_SORTED)
    fms.write_geom_dat(inp, tmp_path / "geom.dat")
    assert (tmp_path / "geom.dat").read_text() == REF_SORTED_GEOM
    rows, iatph = ff.feff_inp_geometry(REF_SORTED)
    assert ff.rdinp_geom_dat_text(rows, iatph) == REF_SORTED_GEOM


def test_reference_first_atom_is_absorber_without_potential_zero(tmp_path):
    text = "TITLE CFAVERAGE smoke\nEDGE K\nCFAVERAGE 1 0 0\nPOTENTIALS\n1 29 Cu\nATOMS\n0.0 0.0 0.0 1 Cu0\n" \
           "1.0 0.0 0.0 1 Cu1\n2.0 0.0 0.0 1 Cu2\nEND\n"
    xyz, ipot, model = fms.geometry_from_feff_inp(_write(tmp_path, text))
    assert list(model) == [1, 2]
    assert ipot[0] == 0 and ipot[1] == 1
    assert np.array_equal(xyz[:, 0], [0.0, 1.0, 2.0])


def _fcc_shells_text(rng, a=3.61, rmax=6.0, absorber_at=(0.3, -0.2, 0.1), comments=True):
    pts = []
    r = int(np.ceil(rmax / a)) + 1
    for i in range(-2 * r, 2 * r + 1):
        for j in range(-2 * r, 2 * r + 1):
            for k in range(-2 * r, 2 * r + 1):
                if (i + j + k) % 2 == 0 and (i * i + j * j + k * k) * (a / 2) ** 2 <= rmax * rmax:
                    pts.append((i * a / 2, j * a / 2, k * a / 2))
    order = rng.permutation(len(pts))
    lines = ["TITLE fcc shells, absorber off the origin", "POTENTIALS", "  0 29 Cu", "  1 29 Cu", "  2 28 Ni", "ATOMS"]
    for n, q in enumerate(order):
        x, y, z = (pts[q][d] + absorber_at[d] for d in range(3))
        if pts[q] == (0.0, 0.0, 0.0):
            ip = 0
        else:
            ip = 1 + (n % 2)
        fx = f"{x:.6f}".replace("e", "D")
        sep = "," if n % 5 == 0 else " "
        tail = f"  Cu{n}  ! inline comment" if comments and n % 3 == 0 else f"  X{n} * ignored after star 9.9"
        lines.append(f"  {fx}{sep}{y:.6f} {z:.6f}   {ip}{tail}")
        if comments and n % 7 == 0:
            lines.append("* a full-line comment inside ATOMS")
    lines.append("END")
    lines.append("1.0 2.0 3.0 1 after-end-is-ignored")
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_fcc_shells_match_oracle_order(tmp_path, seed):
    text = _fcc_shells_text(np.random.default_rng(seed))
    inp = _write(tmp_path, text)
    xyz, ipot, model = fms.geometry_from_feff_inp(inp)
    rows, iatph = ff.feff_inp_geometry(text)
    assert len(rows) == len(ipot) and list(model) == iatph
    assert np.array_equal(xyz, np.array([r[:3] for r in rows]))
    assert list(ipot) == [r[3] for r in rows]
    fms.write_geom_dat(inp, tmp_path / "geom.dat")
    assert (tmp_path / "geom.dat").read_text() == ff.rdinp_geom_dat_text(rows, iatph)
    d = np.einsum("ij,ij->i", xyz, xyz)
    assert np.all(np.diff(d) >= -1e-9)  # non-decreasing distance


def test_fused_distance_decides_near_ties(tmp_path):
    """Two atoms whose distances differ only in the last bit of the fused sum z*z + (x*x + y*y): the order must
    follow the fused value (FEFF's optimised ffsort), which the plain sum would not."""
    rng = np.random.default_rng(3)
    for _ in range(20000):
        x, y, z = (float(v) for v in rng.uniform(0.5, 3.0, 3))
        p, q = (x, y, z), (y, x, z)
        f1, f2 = ff.fma(z, z, ff.fma(x, x, y * y)), ff.fma(z, z, ff.fma(y, y, x * x))
        s1, s2 = x * x + y * y + z * z, y * y + x * x + z * z
        if f1 != f2 and (f1 < f2) != (s1 < s2):
            break
    else:
        pytest.skip("no near tie found")
    far, near = (p, q) if f1 > f2 else (q, p)
    text = "POTENTIALS\n0 29 Cu\n1 29 Cu\nATOMS\n0 0 0 0\n" + \
        f"{far[0]!r} {far[1]!r} {far[2]!r} 1\n{near[0]!r} {near[1]!r} {near[2]!r} 1\nEND\n"
    xyz, _, _ = fms.geometry_from_feff_inp(_write(tmp_path, text))
    assert tuple(xyz[1]) == near and tuple(xyz[2]) == far


def test_rmultiplier_include_and_fortran_exponents(tmp_path):
    _write(tmp_path, "ATOMS\n0.0 0.0 0.0 0\n1.5D0 0.0 0.0 1\n0.0 2.0d0 0.0 1\n", "atoms.inc")
    text = "RMULTIPLIER 2.0\nPOTENTIALS\n0 29 Cu\n1 29 Cu\nINCLUDE atoms.inc\nEND\n"
    xyz, ipot, model = fms.geometry_from_feff_inp(_write(tmp_path, text))
    assert np.array_equal(xyz, [[0, 0, 0], [3.0, 0, 0], [0, 4.0, 0]])
    assert list(ipot) == [0, 1, 1] and list(model) == [1, 2]


def test_coincident_atom_dropped_and_unsupported_inputs(tmp_path):
    text = "POTENTIALS\n0 29 Cu\n1 29 Cu\nATOMS\n1 1 1 1\n1 1 1 0\n1 1 1 1\n2 1 1 1\nEND\n"
    xyz, ipot, _ = fms.geometry_from_feff_inp(_write(tmp_path, text))
    assert len(ipot) == 2 and np.array_equal(xyz[1], [1.0, 0.0, 0.0])
    lat = "LATTICE P 2.0\n1 0 0\n0 1 0\n0 0 1\nPOTENTIALS\n0 29 Cu\nATOMS\n0 0 0 0\nEND\n"
    with pytest.raises(fms.FmsError) as e:
        fms.geometry_from_feff_inp(_write(tmp_path, lat, "lat.inp"))
    assert e.value.code == 13 and "LATTICE" in str(e.value)
    with pytest.raises(fms.FmsError) as e:
        fms.geometry_from_feff_inp(_write(tmp_path, "1 2 3\nATOMS\n", "bad.inp"))
    assert e.value.code == 1
    with pytest.raises(fms.FmsError) as e:
        fms.geometry_from_feff_inp(_write(tmp_path, "POTENTIALS\n0 29 Cu\nATOMS\nEND\n", "empty.inp"))
    assert e.value.code == 2
