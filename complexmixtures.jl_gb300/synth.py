"""Seeded synthetic systems for the benchmark workloads.

No public dataset is involved: every system is generated here from a seed,
with the shapes, sizes and distributions of the five workloads:

  c1  one 1,200-atom self-avoiding chain (1.53 A bonds, >= 3.0 A non-bonded) in a
      60 A cube, 5,000 rigid 3-site waters, 10 frames of sigma 0.5 A jitter,
      cutoff 10 A, binstep 0.02 A, 10 random samples, 120 solute groups of 10 atoms;
  c2  a 20,000-atom random walk confined to a 35 A sphere in a 120 A cube, 50,000
      waters and 2,000 rigid 14-atom cosolvents, sigma 0.5 A, FP32 coordinates,
      cutoff 12 A, 2,000 solute groups of 10 atoms;
  c3  self-MDDF of 10,000 rigid 14-atom molecules in a triclinic cell
      a = b = c = 110 A, alpha = beta = 90, gamma = 60 degrees, sigma 0.4 A, FP32,
      cutoff 10 A, 5 random samples, per-atom groups;
  c4  uneven systems with total atoms log-uniform in [2,000, 200,000], 5 % chain
      solute, the rest water, cubic boxes at 0.1 atoms/A^3;
  c5  c3-like self systems with atoms log-uniform in [5,000, 500,000], 1-200
      frames, cutoff uniform in [8, 14] rounded to the 0.02 A bin step.

Frames jitter the first frame: solute atoms get N(0, sigma) per coordinate;
each rigid solvent molecule gets a rigid displacement (translation
N(0, sigma) per axis and a rotation of angle N(0, sigma / r_g) about a random
axis, r_g its radius of gyration), so molecules stay rigid.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

SEED_BASE = 20261203


def water_template() -> np.ndarray:
    """3-site water: O at the origin, O-H 0.9572 A, H-O-H 104.52 degrees."""
    r, th = 0.9572, math.radians(104.52)
    return np.array([[0.0, 0.0, 0.0], [r, 0.0, 0.0], [r * math.cos(th), r * math.sin(th), 0.0]])


def ball_template(rng: np.random.Generator, n: int, radius: float) -> np.ndarray:
    """n atoms uniform in a ball (seeded internal geometry)."""
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = radius * rng.random(n) ** (1 / 3)
    return d * r[:, None]


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """n uniform random rotation matrices (unit quaternions)."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def small_rotations(rng: np.random.Generator, n: int, sigma_angle: float) -> np.ndarray:
    """Rotations by N(0, sigma_angle) about uniform random axes (Rodrigues)."""
    ax = rng.normal(size=(n, 3))
    ax /= np.linalg.norm(ax, axis=1, keepdims=True)
    ang = rng.normal(scale=sigma_angle, size=n)
    K = np.zeros((n, 3, 3))
    K[:, 0, 1], K[:, 0, 2] = -ax[:, 2], ax[:, 1]
    K[:, 1, 0], K[:, 1, 2] = ax[:, 2], -ax[:, 0]
    K[:, 2, 0], K[:, 2, 1] = -ax[:, 1], ax[:, 0]
    s, c = np.sin(ang)[:, None, None], np.cos(ang)[:, None, None]
    return np.eye(3)[None] + s * K + (1 - c) * (K @ K)


def place_molecules(rng, template: np.ndarray, centres: np.ndarray) -> np.ndarray:
    """Copies of a template at the given centres with random orientations."""
    t = template - template.mean(axis=0)
    R = random_rotations(rng, len(centres))
    return (np.einsum("nij,aj->nai", R, t) + centres[:, None, :]).reshape(-1, 3)


def saw_chain(rng, n: int, bond: float = 1.53, min_sep: float = 3.0, box: Optional[float] = None) -> np.ndarray:
    """Self-avoiding random walk: each new atom at `bond` from the previous one,
    at least `min_sep` from every non-bonded atom (checked with a hash grid)."""
    cell = min_sep
    grid = {}
    pos = np.zeros((n, 3))

    def key(p):
        return (int(math.floor(p[0] / cell)), int(math.floor(p[1] / cell)), int(math.floor(p[2] / cell)))

    def ok(p, i):
        k = key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in grid.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                        if j >= i - 1:
                            continue
                        if np.sum((pos[j] - p) ** 2) < min_sep * min_sep:
                            return False
        return True

    grid.setdefault(key(pos[0]), []).append(0)
    i = 1
    restarts = 0
    while i < n:
        placed = False
        for _ in range(200):
            d = rng.normal(size=3)
            d *= bond / np.linalg.norm(d)
            p = pos[i - 1] + d
            if ok(p, i):
                pos[i] = p
                grid.setdefault(key(p), []).append(i)
                placed = True
                break
        if not placed:  # dead end: step back a few atoms
            back = min(i - 1, 10)
            for j in range(i - back, i):
                grid[key(pos[j])].remove(j)
            i -= back
            restarts += 1
            if restarts > 10000:
                raise RuntimeError("self-avoiding walk failed")
            continue
        i += 1
    return pos - pos.mean(axis=0)


def confined_walk(rng, n: int, radius: float, bond: float = 1.53) -> np.ndarray:
    """Random walk with `bond` steps that never leaves a sphere of `radius`."""
    pos = np.zeros((n, 3))
    for i in range(1, n):
        for _ in range(1000):
            d = rng.normal(size=3)
            p = pos[i - 1] + d * (bond / np.linalg.norm(d))
            if p @ p <= radius * radius:
                pos[i] = p
                break
        else:
            pos[i] = pos[i - 1] * (1 - bond / max(np.linalg.norm(pos[i - 1]), bond))
    return pos


def triclinic_cell(a: float, b: float, c: float, alpha: float, beta: float, gamma: float) -> np.ndarray:
    ca, cb, cg = (math.cos(math.radians(x)) for x in (alpha, beta, gamma))
    sg = math.sin(math.radians(gamma))
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz = math.sqrt(c * c - cx * cx - cy * cy)
    H = np.array([[a, b * cg, cx], [0.0, b * sg, cy], [0.0, 0.0, cz]])
    H[np.abs(H) < 1e-12] = 0.0
    return H


@dataclass
class SolventSpec:
    natomspermol: int
    nmols: int
    frame0: np.ndarray   # [nmols * natomspermol, 3]
    template: np.ndarray
    rg: float


@dataclass
class SynthSystem:
    """One synthetic system: solute frame 0, solvent selections, cell, options."""

    name: str
    cell: np.ndarray                 # [3, 3], columns = lattice vectors
    solute0: np.ndarray              # [Ns, 3]
    solute_nmols: int
    solute_natomspermol: int
    solute_rigid: bool
    solute_template: Optional[np.ndarray]
    solvents: List[SolventSpec]
    cutoff: float
    binstep: float
    n_random_samples: int
    nframes: int
    sigma: float
    seed: int
    solute_group_size: int = 0       # 0 = default per-atom groups
    dtype: type = np.float64
    self_mddf: bool = False

    def frames(self, nframes: Optional[int] = None, solvent: int = 0, start: int = 0):
        """(solute [F, Ns, 3], solvent [F, Nv, 3], cells [F, 3, 3]) for frames
        start .. start+nframes-1 (frame 0 is the unperturbed system)."""
        nframes = self.nframes if nframes is None else nframes
        Ns = len(self.solute0)
        sv = self.solvents[solvent] if self.solvents else None
        xs = np.empty((nframes, Ns, 3), dtype=self.dtype)
        xv = None if self.self_mddf else np.empty((nframes, sv.nmols * sv.natomspermol, 3), dtype=self.dtype)
        for k in range(nframes):
            f = start + k
            rng = np.random.default_rng((self.seed, 7, f))
            if f == 0:
                xs[k] = self.solute0
                if xv is not None:
                    xv[k] = sv.frame0
                continue
            if self.solute_rigid:
                xs[k] = rigid_jitter(rng, self.solute0, self.solute_natomspermol, self.sigma, self._rg_solute())
            else:
                xs[k] = self.solute0 + rng.normal(scale=self.sigma, size=self.solute0.shape)
            if xv is not None:
                rng2 = np.random.default_rng((self.seed, 11 + solvent, f))
                xv[k] = rigid_jitter(rng2, sv.frame0, sv.natomspermol, self.sigma, sv.rg)
        cells = np.repeat(self.cell[None], nframes, axis=0)
        return xs, xv, cells

    def _rg_solute(self) -> float:
        t = self.solute_template - self.solute_template.mean(axis=0)
        return float(np.sqrt((t**2).sum(axis=1).mean()))

    def solute_groups(self):
        """Custom solute groups of `solute_group_size` consecutive atoms, as
        lists of 1-based atom indices (solute atoms are 1..Ns)."""
        if not self.solute_group_size:
            return None
        n = len(self.solute0)
        g = self.solute_group_size
        return [list(range(i + 1, min(i + g, n) + 1)) for i in range(0, n, g)]


def rigid_jitter(rng, x: np.ndarray, apm: int, sigma: float, rg: float) -> np.ndarray:
    m = x.reshape(-1, apm, 3)
    c = m.mean(axis=1, keepdims=True)
    R = small_rotations(rng, len(m), sigma / max(rg, 1e-6))
    t = rng.normal(scale=sigma, size=(len(m), 1, 3))
    return (np.einsum("nij,naj->nai", R, m - c) + c + t).reshape(-1, 3)


def _uniform_in_cell(rng, H, n):
    return rng.random((n, 3)) @ H.T


def _place_rejecting(rng, template, n, H, solute, min_dist):
    """n molecules at uniform centres with random orientations, rejecting
    molecules with an atom closer than min_dist to a solute atom."""
    from scipy.spatial import cKDTree

    L = np.diag(H)
    tree = cKDTree(np.mod(solute, L), boxsize=L) if solute is not None and len(solute) else None
    out = []
    need = n
    while need > 0:
        cand = place_molecules(rng, template, _uniform_in_cell(rng, H, int(need * 1.3) + 16))
        mols = cand.reshape(-1, len(template), 3)
        if tree is not None:
            d, _ = tree.query(np.mod(cand, L))
            okm = (d.reshape(-1, len(template)) >= min_dist).all(axis=1)
            mols = mols[okm]
        out.append(mols[:need])
        need -= len(out[-1])
    return np.concatenate(out).reshape(-1, 3)


def _rg(t):
    t = t - t.mean(axis=0)
    return float(np.sqrt((t**2).sum(axis=1).mean()))


def config1(seed: int = SEED_BASE + 1) -> SynthSystem:
    rng = np.random.default_rng(seed)
    L = 60.0
    H = np.diag([L, L, L])
    solute = saw_chain(rng, 1200) + L / 2
    w = water_template()
    xv = _place_rejecting(rng, w, 5000, H, solute, 2.0)
    return SynthSystem("c1", H, solute, 1, 1200, False, None, [SolventSpec(3, 5000, xv, w, _rg(w))], 10.0, 0.02, 10,
                       10, 0.5, seed, solute_group_size=10)


def config2(seed: int = SEED_BASE + 2, nwater: int = 50000, ncos: int = 2000, nsolute: int = 20000) -> SynthSystem:
    rng = np.random.default_rng(seed)
    L = 120.0
    H = np.diag([L, L, L])
    solute = confined_walk(rng, nsolute, 35.0) + L / 2
    w = water_template()
    xw = place_molecules(rng, w, _uniform_in_cell(rng, H, nwater))
    cos = ball_template(rng, 14, 4.0)
    xc = place_molecules(rng, cos, _uniform_in_cell(rng, H, ncos))
    return SynthSystem("c2", H, solute, 1, nsolute, False, None,
                       [SolventSpec(3, nwater, xw, w, _rg(w)), SolventSpec(14, ncos, xc, cos, _rg(cos))], 12.0, 0.02,
                       10, 1000, 0.5, seed, solute_group_size=10, dtype=np.float32)


def config3(seed: int = SEED_BASE + 3, nmols: int = 10000, edge: float = 110.0, nframes: int = 500) -> SynthSystem:
    rng = np.random.default_rng(seed)
    H = triclinic_cell(edge, edge, edge, 90.0, 90.0, 60.0)
    t = ball_template(rng, 14, 4.0)
    x = place_molecules(rng, t, _uniform_in_cell(rng, H, nmols))
    return SynthSystem("c3", H, x, nmols, 14, True, t, [], 10.0, 0.02, 5, nframes, 0.4, seed, dtype=np.float32,
                       self_mddf=True)


def config4_sizes(seed: int = SEED_BASE + 4, nsystems: int = 64):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(math.log(2000), math.log(200000), nsystems)).astype(int)


def config4_system(natoms: int, seed: int, nframes: int = 50) -> SynthSystem:
    """A c4 system: a chain of 5 % of the atoms (nmols = 1) and water, cubic
    box at 0.1 atoms / A^3."""
    rng = np.random.default_rng(seed)
    nsol = max(10, int(round(0.05 * natoms)))
    nw = max(1, (natoms - nsol) // 3)
    L = ((nsol + 3 * nw) / 0.1) ** (1 / 3)
    H = np.diag([L, L, L])
    solute = confined_walk(rng, nsol, 0.3 * L) + L / 2
    w = water_template()
    xw = place_molecules(rng, w, _uniform_in_cell(rng, H, nw))
    return SynthSystem(f"c4-{natoms}", H, solute, 1, nsol, False, None, [SolventSpec(3, nw, xw, w, _rg(w))], 10.0, 0.02,
                       10, nframes, 0.5, seed, solute_group_size=10, dtype=np.float32)


def config5_request(natoms: int, seed: int, nframes: int) -> SynthSystem:
    """A c5 request: c3-like self system of natoms atoms (14-atom molecules at
    c3 density), cutoff uniform in [8, 14] rounded to a multiple of 0.02."""
    rng = np.random.default_rng(seed)
    nmols = max(2, natoms // 14)
    dens = 10000 / (110.0**3 * math.sin(math.radians(60)))  # molecules / A^3 of c3
    edge = (nmols / dens / math.sin(math.radians(60))) ** (1 / 3)
    H = triclinic_cell(edge, edge, edge, 90.0, 90.0, 60.0)
    t = ball_template(rng, 14, 4.0)
    x = place_molecules(rng, t, _uniform_in_cell(rng, H, nmols))
    cutoff = round(rng.uniform(8.0, 14.0) / 0.02) * 0.02
    cutoff = float(f"{cutoff:.2f}")
    return SynthSystem(f"c5-{natoms}", H, x, nmols, 14, True, t, [], cutoff, 0.02, 5, nframes, 0.4, seed,
                       dtype=np.float32, self_mddf=True)
