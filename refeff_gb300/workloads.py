"""Seeded synthetic FMS workloads with the shapes of the benchmark configurations.

No external dataset is used.  Phase shifts come from a seeded smooth model
t_l(E) (Re delta_l in [-pi, pi], Im delta_l in [0, 0.2]) standing in for the
output of FEFF's xsph stage, which is not available here; clusters are built
from the named lattices.  Energies are complex, Im E = 0.1 eV, and wave
numbers follow k = sqrt(2 (E - E_ref)) / a0 in Angstrom^-1
(crates/refeff-engine/src/fms.rs:4972-4985, a0 = 0.529177249).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

HARTREE_EV = 27.211386
BOHR_ANGSTROM = 0.529177249


@dataclass
class Cluster:
    positions: np.ndarray       # (N, 3) float32, absorber first at the origin
    potentials: np.ndarray      # (N,) int32
    lmaxph: np.ndarray          # (npot,) int32
    name: str = ""

    @property
    def n_atoms(self) -> int:
        return len(self.potentials)

    @property
    def global_lmax(self) -> int:
        return int(self.lmaxph.max())

    @property
    def n_states(self) -> int:
        lm = np.minimum(self.lmaxph[self.potentials], self.global_lmax)
        return int(np.sum((lm + 1) ** 2))


@dataclass
class EnergyGrid:
    energies_ev: np.ndarray     # relative energies (real part), eV
    wave_numbers: np.ndarray    # (E, nsp) complex128, Angstrom^-1
    phase_shifts: np.ndarray    # (E, nsp, 2L+1, npot) complex128
    meta: dict = field(default_factory=dict)


def fcc_sites(a: float, radius: float) -> np.ndarray:
    n = int(np.ceil(radius / a)) + 1
    g = np.arange(-n, n + 1)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    pts = (cells[:, None, :] + basis[None]).reshape(-1, 3) * a
    d = np.linalg.norm(pts, axis=1)
    pts = pts[d <= radius + 1e-9]
    return pts[np.lexsort((pts[:, 2], pts[:, 1], pts[:, 0], np.round(np.linalg.norm(pts, axis=1), 9)))]


def rocksalt_sites(a: float, radius: float):
    """Rocksalt AB: cation on the fcc lattice, anion shifted by (a/2, 0, 0)."""
    n = int(np.ceil(radius / a)) + 1
    g = np.arange(-n, n + 1)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    fcc = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    a_pts = (cells[:, None, :] + fcc[None]).reshape(-1, 3) * a
    b_pts = a_pts + np.array([a / 2, 0, 0])
    pts = np.concatenate([a_pts, b_pts])
    species = np.concatenate([np.zeros(len(a_pts), int), np.ones(len(b_pts), int)])
    keep = np.linalg.norm(pts, axis=1) <= radius + 1e-9
    return pts[keep], species[keep]


def _order(pos, pot):
    d = np.linalg.norm(pos, axis=1)
    idx = np.lexsort((pos[:, 2], pos[:, 1], pos[:, 0], np.round(d, 9)))
    return pos[idx], pot[idx]


def cu_fcc_cluster(radius: float, a: float = 3.61, lmax: int = 3) -> Cluster:
    """fcc Cu around an absorber at the origin: potential 0 absorber, 1 host."""
    pos = fcc_sites(a, radius)
    pot = np.ones(len(pos), np.int32)
    pot[np.argmin(np.linalg.norm(pos, axis=1))] = 0
    pos, pot = _order(pos, pot)
    return Cluster(pos.astype(np.float32), pot.astype(np.int32), np.array([lmax, lmax], np.int32),
                   name=f"fcc Cu a={a} R={radius}")


def displaced_fcc_cluster(rng: np.random.Generator, a: float, radius: float, sigma: float, lmax: int) -> Cluster:
    pos = fcc_sites(a, radius)
    origin = np.argmin(np.linalg.norm(pos, axis=1))
    disp = rng.normal(0.0, sigma, size=pos.shape)
    disp[origin] = 0.0
    pos = pos + disp
    pot = np.ones(len(pos), np.int32)
    pot[origin] = 0
    pos, pot = _order(pos, pot)
    return Cluster(pos.astype(np.float32), pot.astype(np.int32), np.array([lmax, lmax], np.int32),
                   name=f"fcc a={a:.3f} R={radius:.3f} sigma={sigma}")


def rocksalt_cluster(rng: np.random.Generator, a: float = 4.44, radius: float = 9.0, sigma: float = 0.04,
                     lmax: int = 3) -> Cluster:
    pos, species = rocksalt_sites(a, radius)
    origin = np.argmin(np.linalg.norm(pos, axis=1))
    disp = rng.normal(0.0, sigma, size=pos.shape)
    disp[origin] = 0.0
    pos = pos + disp
    pot = np.where(species == 0, 1, 2).astype(np.int32)
    pot[origin] = 0
    pos, pot = _order(pos, pot)
    return Cluster(pos.astype(np.float32), pot, np.array([lmax] * 3, np.int32),
                   name=f"rocksalt a={a} R={radius} sigma={sigma}")


def random_close_packed_cluster(rng: np.random.Generator, n_atoms: int = 600, min_sep: float = 2.2,
                                lmax: int = 4) -> Cluster:
    """Seeded random packing grown outward from the absorber, minimum separation min_sep, 50/50 species."""
    pts = [np.zeros(3)]
    radius = min_sep
    while len(pts) < n_atoms:
        cand = rng.normal(size=(256, 3))
        cand *= (radius * rng.random((256, 1)) ** (1 / 3)) / np.linalg.norm(cand, axis=1, keepdims=True)
        arr = np.asarray(pts)
        for c in cand:
            if np.min(np.linalg.norm(arr - c, axis=1)) >= min_sep:
                pts.append(c)
                arr = np.asarray(pts)
                if len(pts) >= n_atoms:
                    break
        radius *= 1.02
    pos = np.asarray(pts[:n_atoms])
    pot = np.where(rng.random(n_atoms) < 0.5, 1, 2).astype(np.int32)
    pot[0] = 0
    pos, pot = _order(pos, pot)
    return Cluster(pos.astype(np.float32), pot, np.array([lmax] * 3, np.int32), name=f"rcp N={n_atoms}")


def wave_numbers_from_energies(energies_ev: np.ndarray, inner_potential_ev: float = 15.0,
                               broadening_ev: float = 0.1, nsp: int = 1) -> np.ndarray:
    """k = sqrt(2 (E - E_ref)) / a0 with E - E_ref = (E_rel + V0 + i Gamma) in Hartree, narrowed to complex64."""
    e_h = (np.asarray(energies_ev, dtype=np.float64) + inner_potential_ev + 1j * broadening_ev) / HARTREE_EV
    k = np.sqrt(2.0 * e_h) / BOHR_ANGSTROM
    k = k.astype(np.complex64).astype(np.complex128)  # the reference narrows k to Complex32 (fms.rs:4982)
    return np.repeat(k[:, None], nsp, axis=1)


def smooth_phase_shifts(rng: np.random.Generator, wave_numbers: np.ndarray, lmax: int, npot: int,
                        nsp: int = 1) -> np.ndarray:
    """Seeded smooth phase-shift model delta_l(k) per potential, FEFF xphase layout per energy.

    Re delta = a tanh(b |k|) cos(c |k| + d) in [-pi, pi]; Im delta = 0.2 s (1 - exp(-|k|)) in [0, 0.2].
    Entries are stored for signed l = -L..L (index l + L); the +l and -l slots share one model
    (no spin-orbit splitting), as for a non-relativistic xsph run.
    """
    E = wave_numbers.shape[0]
    out = np.zeros((E, nsp, 2 * lmax + 1, npot), np.complex128)
    kabs = np.abs(wave_numbers[:, 0])
    for p in range(npot):
        for l in range(lmax + 1):
            a = rng.uniform(0.4, 2.8) / (1.0 + 0.35 * l)
            b = rng.uniform(0.3, 1.5)
            c = rng.uniform(0.2, 1.2)
            d = rng.uniform(-np.pi, np.pi)
            s = rng.uniform(0.0, 1.0)
            re = np.clip(a * np.tanh(b * kabs) * np.cos(c * kabs + d), -np.pi, np.pi)
            im = 0.2 * s * (1.0 - np.exp(-kabs))
            val = (re + 1j * im).astype(np.complex64).astype(np.complex128)  # narrowed (fms.rs:5049)
            for sp in range(nsp):
                out[:, sp, lmax + l, p] = val
                out[:, sp, lmax - l, p] = val
    return out


def energy_grid(cluster: Cluster, n_energies: int, e_lo: float, e_hi: float, seed: int, nsp: int = 1) -> EnergyGrid:
    rng = np.random.default_rng(seed)
    ev = np.linspace(e_lo, e_hi, n_energies)
    k = wave_numbers_from_energies(ev, nsp=nsp)
    ph = smooth_phase_shifts(rng, k, cluster.global_lmax, len(cluster.lmaxph), nsp)
    return EnergyGrid(ev, k, ph, dict(seed=seed, e_lo=e_lo, e_hi=e_hi))


def xanes_contour(cluster: Cluster, grid: EnergyGrid, n_contour: int = 8, inner_potential_ev: float = 15.0,
                  broadening_ev: float = 0.1, nsp: int = 1):
    """The vertical contour FF2X's xscorr integrates along, appended to a horizontal grid made by energy_grid:
    the Fermi row is the grid energy nearest 0 eV, and the contour runs at that real energy from below the
    broadening down to the real axis (FEFF xsect.dat order: horizontal rows, then the contour, its last row at
    the Fermi level).  The phase shifts of all rows come from one draw of the same seeded model, so the
    horizontal rows equal grid's.  Returns (energies in eV, complex (E + n_contour,), wave numbers, phase
    shifts, Fermi row)."""
    fermi = int(np.argmin(np.abs(grid.energies_ev)))
    ef = float(grid.energies_ev[fermi])
    ims = np.r_[np.linspace(0.15, 0.9, n_contour - 1) * broadening_ev, 0.0]
    k_c = np.concatenate([wave_numbers_from_energies(np.array([ef]), inner_potential_ev, float(y), nsp) for y in ims])
    k_all = np.concatenate([grid.wave_numbers, k_c])
    rng = np.random.default_rng(grid.meta["seed"])
    ph = smooth_phase_shifts(rng, k_all, cluster.global_lmax, len(cluster.lmaxph), nsp)
    ev = np.r_[grid.energies_ev + 1j * broadening_ev, ef + 1j * ims]
    return ev, k_all, ph, fermi


# ---- the named configurations ----

def config0():
    """fcc Cu <= 4.5 A (43 atoms), lmax 3, 100 energies -20..+60 eV (n = 688, m = 16)."""
    cl = cu_fcc_cluster(4.5)
    return cl, energy_grid(cl, 100, -20.0, 60.0, seed=0)


def config1():
    """fcc Cu <= 7.5 A (141 atoms), lmax 3, 200 energies -20..+150 eV (n = 2256, m = 16)."""
    cl = cu_fcc_cluster(7.5)
    return cl, energy_grid(cl, 200, -20.0, 150.0, seed=1)


def config2(n_clusters: int = 32, n_energies: int = 150):
    """32 seeded displaced fcc clusters, a ~ U(3.5, 4.1), R ~ U(4, 7), lmax in {2, 3}, 150 energies each."""
    rng = np.random.default_rng(2)
    out = []
    for c in range(n_clusters):
        a = rng.uniform(3.5, 4.1)
        r = rng.uniform(4.0, 7.0)
        lmax = int(rng.integers(2, 4))
        cl = displaced_fcc_cluster(rng, a, r, 0.05, lmax)
        out.append((cl, energy_grid(cl, n_energies, -20.0, 60.0, seed=1000 + c)))
    return out


def config3():
    """Rocksalt AB a=4.44 A, sigma 0.04, R 9 A (~280 atoms), 3 potentials, lmax 3, 300 energies."""
    rng = np.random.default_rng(3)
    cl = rocksalt_cluster(rng)
    return cl, energy_grid(cl, 300, -20.0, 100.0, seed=3)


def config4():
    """Random close packed 600 atoms, 50/50 species, lmax 4 (n = 15000), 400 energies -20..+300 eV."""
    rng = np.random.default_rng(4)
    cl = random_close_packed_cluster(rng)
    return cl, energy_grid(cl, 400, -20.0, 300.0, seed=4)


def small_cluster(radius: float = 3.0, lmax: int = 2, n_energies: int = 6, seed: int = 7, nsp: int = 1):
    """A small fcc cluster for quick parity checks (oracle runs in well under a second)."""
    cl = cu_fcc_cluster(radius, lmax=lmax)
    return cl, energy_grid(cl, n_energies, -10.0, 40.0, seed=seed, nsp=nsp)
