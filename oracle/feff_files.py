"""TEST INFRASTRUCTURE ONLY: FEFF handoff files for the file-seam tests.

Restates, independently of the product, the reference's writers for the
files the `fms` stage reads (phase.bin with its PAD encoding, fms.inp,
global.inp, geom.dat) and the gg.dat text it writes, so that tests can build
FEFF work directories and check the product's gg.bin / gg.dat byte for byte.

  PAD encode/decode   crates/refeff-io/src/pad.rs:33-127
  Fortran E20.10      crates/refeff-io/src/format.rs:164-209
  gg.dat text         crates/refeff-io/src/gg_dat.rs:155-233
  phase.bin text      crates/refeff-io/src/phase_bin/render.rs:14-99
  fms.inp text        crates/refeff-io/src/fms_input.rs:214-246
  global.inp text     crates/refeff-io/src/global_input.rs:108-190
  geom.dat text       crates/refeff-io/src/structure_output.rs:204-223
  fms.bin text        crates/refeff-io/src/fms_bin.rs:77-98
  gtr.dat text        crates/refeff-io/src/gtr_dat.rs:60-71
  gg_slice.bin        crates/refeff-io/src/rhorrp_gg_bin.rs:99-160
  gg_diag.bin         crates/refeff-io/src/rhorrp_gg_bin.rs:178-252
  feff.inp -> geom    crates/refeff-io/src/input.rs:146-372 (lines, comments, BWORDS),
                      crates/refeff-io/src/model.rs:626-676 (ATOMS / POTENTIALS rows),
                      crates/refeff-io/src/rdinp/geometry.rs:18-119 (rows, ffsort, iatph),
                      crates/refeff-io/src/rdinp/structure.rs:57-81 (write_geom_dat)
"""
from __future__ import annotations

import math
from fractions import Fraction
from pathlib import Path

import numpy as np

IOFF, IBASE, IHUGE, IBAS2 = 37, 90, 38, 45
TENLOG = 2.3025850929940455


def powi(a: float, b: int) -> float:
    """Integer power by repeated squaring (what the reference's powi lowers to)."""
    recip = b < 0
    r = 1.0
    while True:
        if b & 1:
            r *= a
        b = int(b / 2)  # truncation toward zero, like C integer division
        if b == 0:
            break
        a *= a
    return 1.0 / r if recip else r


def _trunc(x: float) -> int:
    return int(x)  # Rust `as i32` truncates toward zero


def pad_encode(value: float, npack: int) -> str:
    huge = powi(10.0, IHUGE)
    tiny = 1.0 / huge
    out = [ord(" ")] * npack
    xsave = min(max(value, -huge), huge)
    isgn = 1 if xsave > 0.0 else 0
    xwork = abs(xsave)
    iexp = 0
    if tiny < xwork < huge:
        iexp = 1 + _trunc(math.log(xwork) / TENLOG)
    elif xwork >= huge:
        iexp = IHUGE
        xwork = 1.0
    elif xwork <= tiny:
        xwork = 0.0
    xwork /= powi(10.0, iexp)
    while True:
        if xwork >= 1.0:
            xwork *= 0.1
            iexp += 1
        elif xwork <= 0.099999999994:
            xwork *= 10.0
            iexp -= 1
        if xwork < 1.0:
            break
    itmp = _trunc(float(IBAS2) * xwork)
    out[0] = iexp + IOFF + IBAS2
    out[1] = 2 * itmp + isgn + IOFF
    xwork = xwork * float(IBAS2) - float(itmp)
    for slot in range(2, npack):
        itmp = _trunc(float(IBASE) * xwork + 1.0e-9)
        out[slot] = itmp + IOFF
        xwork = xwork * float(IBASE) - float(itmp)
    if xwork >= 0.5:
        rounded = itmp + IOFF + 1
        if rounded <= 126:
            out[npack - 1] = rounded
        elif out[npack - 2] < 126:
            out[npack - 2] += 1
            out[npack - 1] = 37
    return bytes(out).decode("ascii")


def pad_decode(s: str, npack: int) -> float:
    b = s.encode("ascii")
    iexp = b[0] - IOFF - IBAS2
    second = b[1] - IOFF
    isgn = (second % 2) * 2 - 1
    itmp = second // 2
    base = float(IBASE)
    total = float(itmp) / powi(base, 2)
    for i in range(npack - 1, 1, -1):
        total += float(b[i] - IOFF) / powi(base, i + 1)
    return 2.0 * float(isgn) * float(IBASE) * total * powi(10.0, iexp)


def encode_reals(values, npack: int) -> str:
    out, payload = [], ""
    maxp = 82 - npack + 1
    for i, v in enumerate(values):
        payload += pad_encode(float(v), npack)
        if len(payload) >= maxp or i == len(values) - 1:
            out.append("!" + payload)
            payload = ""
    return "".join(line + "\n" for line in out)


def encode_complex(values, npack: int) -> str:
    out, payload = [], ""
    maxp = 82 - 2 * npack + 1
    for i, v in enumerate(values):
        payload += pad_encode(float(v.real), npack) + pad_encode(float(v.imag), npack)
        if len(payload) >= maxp or i == len(values) - 1:
            out.append("$" + payload)
            payload = ""
    return "".join(line + "\n" for line in out)


def fortran_exp(value: float, width: int = 20, precision: int = 10, min_exp_width: int = 2) -> str:
    exponent = 0 if value == 0.0 else math.floor(math.log10(abs(value))) + 1
    mantissa = value if value == 0.0 else value / powi(10.0, exponent)
    m = f"{mantissa:.{precision}f}"
    digits = str(abs(exponent))
    ew = max(len(digits), min_exp_width)
    field = len(m) + 2 + ew
    return " " * max(0, width - field) + m + "E" + ("-" if exponent < 0 else "+") + digits.zfill(ew)


def gg_dat_text(sections) -> str:
    """sections: list of square complex arrays (row, column)."""
    out = []
    for number, sec in enumerate(sections, start=1):
        r, c = sec.shape
        out.append(f"#SN#   Section: {number:4d}\n")
        out.append("#DF# This section written in txt.\n#H#\n")
        out.append(f"#DT# 2D complex array with sizes {r:4d}{c:4d}\n")
        out.append("#H# File is organized as follows:  Array(1,i)     Array(1,i+1)    Array(1,i+2)  . . .\n")
        out.append("#H#                                Array(2,i)\n")
        out.append("#H#                                     .\n" * 3)
        for row in range(r):
            out.append("".join(fortran_exp(float(v.real)) + " " + fortran_exp(float(v.imag)) for v in sec[row]) + "\n")
    return "".join(out)


def parse_gg_dat(text: str):
    sections, cur, dim = [], [], 0
    for line in text.splitlines():
        if line.startswith("#DT#"):
            dim = int(line[-8:-4])
            cur = []
        elif line.startswith("#"):
            continue
        elif line.strip():
            vals = [float(line[i:i + 20]) for i in range(0, len(line), 41)]
            ims = [float(line[i + 21:i + 41]) for i in range(0, len(line), 41)]
            cur.append(np.array(vals) + 1j * np.array(ims))
            if len(cur) == dim:
                sections.append(np.array(cur))
    return sections


def _record(payload: bytes) -> bytes:
    """One Fortran sequential unformatted record: u32 length, payload, u32 length (little-endian)."""
    n = len(payload).to_bytes(4, "little")
    return n + payload + n


def gg_slice_bin_bytes(values) -> bytes:
    """gg_slice.bin from (energy, row, column) complex values (rhorrp_gg_slice_bin_bytes, rhorrp_gg_bin.rs:138-160):
    header (ldim, istate, ne) as i32, then complex64 in energy / column / row order."""
    v = np.asarray(values, dtype=np.complex64)
    ne, rows, cols = v.shape
    header = np.array([rows, cols, ne], dtype="<i4").tobytes()
    return _record(header) + _record(v.transpose(0, 2, 1).astype("<c8").tobytes())


def gg_diag_bin_bytes(values) -> bytes:
    """gg_diag.bin from (energy, atom, row, column) values (rhorrp_gg_diag_bin_bytes, rhorrp_gg_bin.rs:228-252):
    header (ldim, ldim, inclus, ne) as i32, then complex64 in energy / atom / column / row order."""
    v = np.asarray(values, dtype=np.complex64)
    ne, na, dim, _ = v.shape
    header = np.array([dim, dim, na, ne], dtype="<i4").tobytes()
    return _record(header) + _record(v.transpose(0, 1, 3, 2).astype("<c8").tobytes())


def _records(data: bytes):
    out, pos = [], 0
    while pos < len(data):
        n = int.from_bytes(data[pos:pos + 4], "little")
        out.append(data[pos + 4:pos + 4 + n])
        if data[pos + 4 + n:pos + 8 + n] != data[pos:pos + 4]:
            raise ValueError("record markers differ")
        pos += 8 + n
    return out


def parse_gg_slice_bin(data: bytes):
    """(energy, row, column) complex64 array from gg_slice.bin bytes (parse_rhorrp_gg_slice_bin, :99-136)."""
    header, payload = _records(data)
    rows, cols, ne = np.frombuffer(header, dtype="<i4")
    return np.frombuffer(payload, dtype="<c8").reshape(ne, cols, rows).transpose(0, 2, 1)


def parse_gg_diag_bin(data: bytes):
    """(energy, atom, row, column) complex64 array from gg_diag.bin bytes (parse_rhorrp_gg_diag_bin, :178-226)."""
    header, payload = _records(data)
    dim, dim2, na, ne = np.frombuffer(header, dtype="<i4")
    if dim != dim2:
        raise ValueError("gg_diag ldim values differ")
    return np.frombuffer(payload, dtype="<c8").reshape(ne, na, dim, dim).transpose(0, 1, 3, 2)


def phase_bin_text(*, nsp, energy_grid, reference_energy, potentials, pad_width=8, transition_count=8,
                   edge=8979.0) -> str:
    """potentials: list of (lmax, iz, label, phase array (ne, 2lmax+1, nsp))."""
    ne = len(energy_grid)
    hdr = [nsp, ne, ne, 0, len(potentials) - 1, 1, 1, pad_width, transition_count, transition_count, 1]
    out = "".join(f" {v:>4d}" for v in hdr) + "\n"
    out += encode_reals([1.2, 0.0, edge], pad_width)
    out += encode_complex(list(energy_grid), pad_width)
    eref = np.asarray(reference_energy).reshape(ne, nsp)
    out += encode_complex([eref[e, s] for s in range(nsp) for e in range(ne)], pad_width)
    for lmax, iz, label, ph in potentials:
        out += f" {lmax:>3d} {iz:>3d} {label:<6s}\n"
        for s in range(nsp):
            out += encode_complex([ph[e, l, s] for e in range(ne) for l in range(2 * lmax + 1)], pad_width)
    rkk = [complex(0.2 + 0.03 * e + 0.015 * t, -0.01 * t) for s in range(nsp) for t in range(transition_count)
           for e in range(ne)]
    out += encode_complex(rkk, pad_width)
    return out


def fms_inp_text(*, lmaxph, rfms2, rdirec, toler1=1e-3, toler2=1e-3, idwopt=-1, sig2g=0.0, minv=0, mfms=1,
                 do_fms=0, save_gg_slice=False, tk=0.0, thetad=0.0) -> str:
    def i4(vals):
        return "".join(f"{v:4d}" for v in vals)
    return ("mfms, idwopt, minv\n" + i4([mfms, idwopt, minv]) + "\n"
            "rfms2, rdirec, toler1, toler2\n" + f"{rfms2:13.5f}{rdirec:13.5f}{toler1:13.5f}{toler2:13.5f}\n"
            "tk, thetad, sig2g\n" + f"{tk:13.5f}{thetad:13.5f}{sig2g:13.5f}\n"
            " lmaxph(0:nph)\n" + i4(lmaxph) + "\n"
            " the number of decomposi\n" + f"{-1:5d}\n"
            " save_gg_slice\n" + ("T" if save_gg_slice else "F") + "\n"
            "do_fms\n" + i4([do_fms]) + "\n")


def global_inp_text(ispin: int = 0, *, ipol: int = 0, le2: int = 0, elpty: float = 0.0, angks: float = 0.0,
                    do_nrixs: int = 0, polarization_tensor=None) -> str:
    """global.inp (crates/refeff-io/src/global_input.rs:108-190) with one q vector; polarization_tensor is 3x3
    complex (rows m = -1, 0, 1), written as 3 rows of 6 F13.5 fields."""
    ptz = np.zeros((3, 3), complex) if polarization_tensor is None else np.asarray(polarization_tensor, complex)
    out = " nabs, iphabs - CFAVERAGE data\n" + f"{1:8d}{0:8d}{0.0:13.5f}\n"
    out += " ipol, ispin, le2, elpty, angks, l2lp, do_nrixs, ldecmx, lj\n"
    out += f"{ipol:5d}{ispin:5d}{le2:5d}{elpty:12.4f}{angks:12.4f}{0:5d}{do_nrixs:5d}{-1:5d}{0:5d}\n"
    out += "evec\t\t  xivec \t   spvec\n"
    out += "".join(f"{a:13.5f}{b:13.5f}{c:13.5f}\n" for a, b, c in [(0, 1, 0), (0, 0, 0), (1, 0, 1)])
    out += " polarization tensor \n"
    for r in range(3):
        out += "".join(f"{v:13.5f}" for z in ptz[r] for v in (z.real, z.imag)) + "\n"
    out += "evnorm, xivnorm, spvnorm - only used for nrixs\n" + f"{0.0:13.5f}{0.0:13.5f}{0.0:13.5f}\n"
    out += "nq,    imdff,   qaverage,   mixdff\n" + f"{1:12d}{0:12d} F F\n"
    out += " q-vectors : qx, qy, qz, q(norm), weight, qcosth, qsinth, qcosfi, qsinfi\n"
    out += "".join(f"{v:13.5f}" for v in [0, 0, 0, 0, 1, 0, 1, 0, 0, 1]) + "\n"
    return out


def fms_bin_text(traces, *, cluster_radius, ne1=None, ne3=0, nph, pad_width=8) -> str:
    """fms.bin (crates/refeff-io/src/fms_bin.rs:77-98); traces (n_spectra, ne)."""
    tr = np.asarray(traces, complex)
    ne = tr.shape[1]
    counts = [ne, ne if ne1 is None else ne1, ne3, nph, pad_width, 0]
    out = f"FMS rfms={cluster_radius:7.4f}\n" + "".join(f" {c:>7d}" for c in counts) + "\n"
    for row in tr:
        out += encode_complex(list(row), pad_width)
    return out


def parse_fms_bin(text: str):
    """Title radius, counts and the decoded spectra (n_spectra, ne) of an fms.bin."""
    lines = text.splitlines()
    radius = float(lines[0].split("=")[1])
    counts = [int(x) for x in lines[1].split()]
    ne, npad = counts[0], counts[4]
    vals = []
    for line in lines[2:]:
        p = line[1:]
        for k in range(0, len(p), 2 * npad):
            vals.append(complex(pad_decode(p[k:k + npad], npad), pad_decode(p[k + npad:k + 2 * npad], npad)))
    return radius, counts, np.array(vals).reshape(-1, ne) if ne else np.zeros((0, 0), complex)


def gtr_dat_text(energy, trace) -> str:
    """gtr.dat (crates/refeff-io/src/gtr_dat.rs:60-71)."""
    return "".join(f"{e.real:13.6f}{e.imag:13.6f}{t.real:13.6f}{t.imag:13.6f}\n" for e, t in zip(energy, trace))


def read_rkk(phase_bin: str, *, nsp, ne, ntrans=8):
    """The q = 0 transition moments (ne, ntrans, nsp) of a phase.bin written by phase_bin_text: the last block."""
    lines = phase_bin.splitlines()
    npad = int(lines[0].split()[7])
    per_line = (82 - 2 * npad + 1 + 2 * npad - 1) // (2 * npad)
    count = ne * ntrans * nsp
    nlines = -(-count // per_line)
    vals = []
    for line in lines[-nlines:]:
        p = line[1:]
        for k in range(0, len(p), 2 * npad):
            vals.append(complex(pad_decode(p[k:k + npad], npad), pad_decode(p[k + npad:k + 2 * npad], npad)))
    return np.array(vals[:count]).reshape((ne, ntrans, nsp), order="F")


def geom_dat_text(positions, potentials) -> str:
    nph = int(max(potentials))
    out = f"nat, nph = {len(potentials):5d}{nph:5d}\n"
    out += "".join(f"{i + 1:5d}" for i in range(nph + 1)) + "\n"
    out += " iat     x       y        z       iph  \n " + "-" * 71 + "\n"
    for i, (p, ip) in enumerate(zip(positions, potentials)):
        out += f"{i + 1:4d}{p[0]:13.5f}{p[1]:13.5f}{p[2]:13.5f}{int(ip):4d}{0:4d}\n"
    return out


def write_workdir(path: Path, *, positions, potentials, lmaxph, energy_grid, phase_potentials, nsp=1, ispin=0,
                  rfms2=100.0, rdirec=100.0, sig2g=0.0, do_fms=0, nspu=None, global_kw=None, idwopt=-1, tk=0.0,
                  thetad=0.0):
    path.mkdir(parents=True, exist_ok=True)
    ne = len(energy_grid)
    (path / "phase.bin").write_text(phase_bin_text(nsp=nsp, energy_grid=energy_grid,
                                                   reference_energy=np.zeros((ne, nsp), complex),
                                                   potentials=phase_potentials))
    (path / "fms.inp").write_text(fms_inp_text(lmaxph=lmaxph, rfms2=rfms2, rdirec=rdirec, sig2g=sig2g,
                                               do_fms=do_fms, idwopt=idwopt, tk=tk, thetad=thetad))
    (path / "global.inp").write_text(global_inp_text(ispin, **(global_kw or {})))
    (path / "geom.dat").write_text(geom_dat_text(positions, potentials))
    if nspu is not None:
        (path / ".dimensions.dat").write_text(f"{300:12d}{max(lmaxph):12d}{len(lmaxph) - 1:12d}{nspu:12d}\n")


def reference_engine_fixture(path: Path):
    """The reference engine's FMS source fixture (crates/refeff-engine/src/fms/tests.rs:2381-2421, 2501-2525,
    2821-2875): two atoms 1.4 A apart, two energies, two potentials with lmax 2, lmaxph [1, 1], rfms2 3, rdirec 5,
    K edge (ihole 1), isotropic global.inp (ipol 0, ispin 0, le2 0, polarization tensor diag(1/3))."""
    grid = [complex(1.0, 0.02), complex(1.4, 0.03)]
    pots = []
    for p in range(2):
        ph = np.zeros((2, 5, 1), complex)
        for e in range(2):
            for sl in range(5):
                ph[e, sl, 0] = complex(0.03 * (p + 1) + 0.01 * e + 0.02 * sl, 0.004 * (sl + 1))
        pots.append((2, 29, "Cu", ph))
    write_workdir(path, positions=[[0, 0, 0], [1.4, 0, 0]], potentials=[0, 1], lmaxph=[1, 1], energy_grid=grid,
                  phase_potentials=pots, rfms2=3.0, rdirec=5.0,
                  global_kw={"polarization_tensor": np.eye(3) / 3.0})


# ---- feff.inp -> geometry rows (rdinp) ----

_BLOCKS = {"ATOMS", "POTENTIALS", "OVERLAP", "LATTICE", "EGRID", "DENSITY", "CONFIG", "STRETCHES", "ANGLES", "ELNES",
           "EXELFS", "NRIXS", "MDFF"}
_CANON = {"ATOM": "ATOMS", "CONF": "CONFIG", "DENS": "DENSITY", "ELNE": "ELNES", "EXEL": "EXELFS", "EGRI": "EGRID",
          "LATT": "LATTICE", "MDFF": "MDFF", "NRIX": "NRIXS", "OVER": "OVERLAP", "POTE": "POTENTIALS", "TITL": "TITLE"}


def fma(a: float, b: float, c: float) -> float:
    """Correctly rounded a*b + c (the exact value through rationals, rounded once)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _strip_inline(line: str) -> str:
    opens, closes = "[{\"'(", "]}\"')"
    prot = None
    for i, ch in enumerate(line):
        if prot is not None:
            if ch == closes[prot]:
                prot = None
            continue
        if ch in opens:
            prot = opens.index(ch)
            continue
        if ch in "!#%":
            return line[:i]
    return line


def _bwords(line: str):
    words, start, comma = [], None, True
    for i, ch in enumerate(line):
        if ch in " \t":
            if start is not None:
                words.append(line[start:i])
                start, comma = None, False
        elif ch == ",":
            if start is not None:
                words.append(line[start:i])
                start = None
            elif comma:
                words.append("")
            comma = True
        elif start is None:
            start = i
    if start is not None:
        words.append(line[start:].rstrip())
    return words


def feff_inp_lines(text: str):
    """(is_card, keyword_or_section, fields) per logical line, stopping after END (no INCLUDE here)."""
    out, active = [], None
    for raw in text.splitlines():
        t = raw.replace("\t", " ").lstrip()
        if not t or t[0] in ";*%#":
            continue
        u = _strip_inline(t).strip()
        if not u:
            continue
        tok = _bwords(u)
        if not tok:
            continue
        first = tok[0]
        payload = (active == "EGRID" and first.lower() in ("e_grid", "k_grid", "exp_grid", "user_grid")) or \
                  (active == "DENSITY" and first.lower() in ("line", "plane", "volume"))
        if not payload and first[:1].isascii() and first[:1].isalpha():
            key = first.upper()
            key = _CANON.get(key[:4], key)
            out.append((True, key, tok[1:]))
            if key == "END":
                break
            if key in _BLOCKS:
                active = key
            elif key != "TITLE":
                active = None
        elif active is not None:
            out.append((False, active, tok))
        else:
            raise ValueError("data row found outside a block card")
    return out


def _f64(v: str) -> float:
    return float(v.replace("D", "E").replace("d", "E"))


def feff_inp_geometry(text: str):
    """(rows, iatph): rows = [(x, y, z, ipot)] in geom.dat order, iatph one-based model atoms."""
    lines = feff_inp_lines(text)
    rmult = None
    atoms, pots = [], []
    for card, key, f in lines:
        if card:
            if rmult is None and (key == "RMULT" or key[:4] == "RMUL"):
                rmult = _f64(f[0])
            continue
        f = f[:f.index("*")] if "*" in f else f
        if key == "ATOMS":
            atoms.append([_f64(f[0]), _f64(f[1]), _f64(f[2]), int(f[3])])
        elif key == "POTENTIALS":
            int(f[1])
            pots.append(int(f[0]))
    rmult = 1.0 if rmult is None else rmult
    atoms = [[a[0] * rmult, a[1] * rmult, a[2] * rmult, a[3]] for a in atoms]
    ia = next((i for i, a in enumerate(atoms) if a[3] == 0), 0)
    c = atoms[ia]
    rows = [(0.0, 0.0, 0.0, 0, 0.0)]
    for i, a in enumerate(atoms):
        if i == ia:
            continue
        x, y, z = a[0] - c[0], a[1] - c[1], a[2] - c[2]
        d2 = fma(z, z, fma(x, x, y * y))
        if d2 > 0.0:
            rows.append((x, y, z, a[3], d2))
    for i in range(len(rows) - 1):
        mi, md = i, rows[i][4]
        for j in range(i + 1, len(rows)):
            if rows[j][4] < md:
                mi, md = j, rows[j][4]
        if mi != i:
            rows[i], rows[mi] = rows[mi], rows[i]
    maxp = max((max(p, 0) for p in pots), default=None)
    if maxp is None:
        maxp = max(max(r[3], 0) for r in rows)
    iatph = [0] * (maxp + 1)
    iatph[0] = 1
    for iph in range(1, maxp + 1):
        iatph[iph] = next((k + 1 for k, r in enumerate(rows) if r[3] == iph), 0)
    while len(iatph) > 1 and iatph[-1] == 0:
        iatph.pop()
    return [r[:4] for r in rows], iatph


def rdinp_geom_dat_text(rows, iatph) -> str:
    """write_geom_dat (crates/refeff-io/src/rdinp/structure.rs:57-81)."""
    out = f"nat, nph = {len(rows):5d}{len(iatph) - 1:5d}\n" + "".join(f"{m:5d}" for m in iatph) + "\n"
    out += " iat     x       y        z       iph  \n " + "-" * 71 + "\n"
    for i, r in enumerate(rows):
        out += f"{i + 1:4d}{r[0]:13.5f}{r[1]:13.5f}{r[2]:13.5f}{r[3]:4d}{1:4d}\n"
    return out
