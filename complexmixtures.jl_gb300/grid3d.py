"""grid3D (src/tools/grid3D.jl:47-152): a grid of points around the solute,
each labelled with its closest solute atom and that atom's contribution to the
MDDF (or coordination number, or md count) at the point's distance, written
as a PDB whose atoms are the grid points (occupancy = distance, beta = scaled
contribution).  The grid search runs on the GPU (cm_grid3d); the per-atom
contribution curves, the scaling and the PDB output are host-side.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _native as N
from .results import Result


@dataclass
class Atoms:
    """The atoms of a structure, indexed by the 1-based indices of the
    AtomSelections: coordinates [N, 3] and optional per-atom labels (the
    PDBTools.Atom fields grid3D copies into its output)."""

    xyz: np.ndarray
    name: List[str] = field(default_factory=list)
    resname: List[str] = field(default_factory=list)
    chain: List[str] = field(default_factory=list)
    resnum: List[int] = field(default_factory=list)
    element: List[str] = field(default_factory=list)
    index: List[int] = field(default_factory=list)   # 1-based atom indices (PDBTools.index); default 1..N

    def __post_init__(self):
        self.xyz = np.asarray(self.xyz, dtype=np.float64).reshape(-1, 3)
        n = len(self.xyz)
        self.index = [int(i) for i in self.index] or list(range(1, n + 1))
        self.name = list(self.name) or ["X"] * n
        self.resname = list(self.resname) or ["UNK"] * n
        self.chain = list(self.chain) or ["A"] * n
        self.resnum = [int(r) for r in self.resnum] or [1] * n
        self.element = list(self.element) or [""] * n

    def take(self, keep) -> "Atoms":
        """The atoms at the given positions, or where a boolean mask is true,
        keeping their indices (a PDBTools selection of the structure)."""
        keep = np.asarray(keep)
        pos = np.nonzero(keep)[0] if keep.dtype == bool else keep.astype(np.int64)
        pick = lambda v: [v[int(k)] for k in pos]
        return Atoms(self.xyz[pos], pick(self.name), pick(self.resname), pick(self.chain), pick(self.resnum),
                     pick(self.element), pick(self.index))


def read_pdb_atoms(path: str) -> Atoms:
    """ATOM / HETATM records of the first model of a PDB file."""
    xyz, name, resname, chain, resnum, element = [], [], [], [], [], []
    with open(path) as f:
        for line in f:
            if line.startswith(("ENDMDL", "END")) and xyz:
                break
            if line.startswith(("ATOM", "HETATM")):
                name.append(line[12:16].strip())
                resname.append(line[17:21].strip())
                chain.append(line[21:22].strip() or "A")
                resnum.append(int(line[22:26]))
                xyz.append((float(line[30:38]), float(line[38:46]), float(line[46:54])))
                element.append(line[76:78].strip() if len(line) >= 78 else "")
    return Atoms(np.array(xyz), name, resname, chain, resnum, element)


@dataclass
class Grid3D:
    """Kept grid points in ascending grid order: position, the closest solute
    atom (1-based index into the structure), its distance (PDB occupancy),
    the interpolated contribution and that contribution scaled to [0, 1] over
    the grid (PDB beta), with the closest atom's labels."""

    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    index: np.ndarray
    occup: np.ndarray
    value: np.ndarray
    beta: np.ndarray
    name: List[str]
    resname: List[str]
    chain: List[str]
    resnum: List[int]
    element: List[str]
    n: tuple
    origin: np.ndarray

    def __len__(self) -> int:
        return len(self.x)

    def write_pdb(self, path: str) -> None:
        with open(path, "w") as f:
            for k in range(len(self)):
                nm = self.name[k]
                nm = nm if len(nm) >= 4 else " " + nm
                f.write("ATOM  %5d %-4s %3s %1s%4d    %8.3f%8.3f%8.3f%6.2f%6.2f          %2s\n" % (
                    (k + 1) % 100000, nm[:4], self.resname[k][:3], self.chain[k][:1], self.resnum[k] % 10000,
                    self.x[k], self.y[k], self.z[k], self.occup[k], self.beta[k], self.element[k][:2]))
            f.write("END\n")


def atom_contribution_table(result: Result, type: str = "mddf") -> np.ndarray:
    """Contribution curve of each atom type of the solute molecule: the
    values of ``contributions(result, SoluteGroup([atom]), type=type)``
    (src/tools/grid3D.jl:97, src/tools/contributions.jl:70-248) for every
    atom at once, with the same arithmetic (a one-atom group's row, divided
    by nmols when the selection has several molecules)."""
    sel = result.solute
    gc = np.asarray(result.solute_group_count, dtype=np.float64)[: sel.natomspermol]
    rows = np.zeros_like(gc) + (gc if sel.nmols == 1 else gc / sel.nmols)
    if type == "mddf":
        mdr = np.asarray(result.md_count_random, dtype=np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(mdr == 0.0, 0.0, rows / np.where(mdr == 0.0, 1.0, mdr))
    if type == "coordination_number":
        return np.add.accumulate(rows, axis=1)
    if type == "md_count":
        return rows
    raise ValueError("type must be :mddf, :coordination_number or :md_count")


def grid3D(result: Result, atoms: Atoms, output_file: Optional[str] = None, *, dmin: float = 1.5, dmax: float = 5.0,
           step: float = 0.5, silent: bool = False, type: str = "mddf", device: int = 0) -> Grid3D:
    """src/tools/grid3D.jl:47-152 (the grid search on the GPU)."""
    if result.solute.custom_groups:
        raise ValueError("The 3D grid can only be built if the contributions of all atoms of the solute are recorded. "
                         "It is not compatible with predefined groups of atoms.")
    if type not in ("mddf", "coordination_number", "md_count"):
        raise ValueError("type must be :mddf, :coordination_number or :md_count")
    sel = result.solute
    idx = np.asarray(sel.indices, dtype=np.int64)
    xyz = atoms.xyz[idx - 1]
    atype = (idx - idx[0]) % sel.natomspermol
    point, atom, dist, val, n, origin = grid_search(xyz, atype, atom_contribution_table(result, type), result.d,
                                                    dmin=dmin, dmax=dmax, step=step, device=device)
    k = len(point)
    ix, rem = np.divmod(point, n[1] * n[2])
    iy, iz = np.divmod(rem, n[2])
    pos = [origin[a] + step * i.astype(np.float64) for a, i in enumerate((ix, iy, iz))]
    # beta scaled to [0, 1] over the kept points (src/tools/grid3D.jl:139-146)
    bmin, bmax = (val.min(), val.max()) if k else (0.0, 1.0)
    beta = (val - bmin) / (bmax - bmin) if k else val
    gi = idx[atom] if k else np.zeros(0, dtype=np.int64)
    g = Grid3D(pos[0], pos[1], pos[2], gi, dist, val, beta, [atoms.name[i - 1] for i in gi],
               [atoms.resname[i - 1] for i in gi], [atoms.chain[i - 1] for i in gi], [atoms.resnum[i - 1] for i in gi],
               [atoms.element[i - 1] for i in gi], n, origin)
    if output_file is not None:
        g.write_pdb(output_file)
        if not silent:
            print(f"Grid written to {output_file}")
    return g


def grid_search(xyz, atom_type, table, d, *, dmin: float, dmax: float, step: float, device: int = 0):
    """The grid search of grid3D on the GPU (cm_grid3d): every point of the
    grid around the atoms ``xyz`` whose closest atom lies between dmin and
    dmax, with that atom's contribution curve ``table[atom_type[atom]]``
    (over the distances ``d``) interpolated at the distance, kept when
    positive.  Returns, in ascending grid order, the points' linear indices,
    the closest atoms (0-based), the distances and the values, plus the grid
    shape and origin."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    atype = np.ascontiguousarray(np.asarray(atom_type).astype(np.int32))
    table = np.ascontiguousarray(table, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    lib = N.load()
    desc = N.cm_grid3d_desc(device=device, nbins=len(d), natoms=len(xyz), ntypes=table.shape[0], dmin=dmin,
                            dmax=dmax, step=step)
    desc.xyz = N.as_ptr(xyz, C.c_double)
    desc.atom_type = N.as_ptr(atype, C.c_int32)
    desc.table = N.as_ptr(table, C.c_double)
    desc.d = N.as_ptr(d, C.c_double)
    out = N.cm_grid3d_out()
    xmin, xmax = xyz.min(axis=0), xyz.max(axis=0)
    cap = int(np.prod([np.ceil((xmax[k] - xmin[k] + 2 * dmax) / step + 1) for k in range(3)]))
    point = np.zeros(cap, dtype=np.int64)
    atom = np.zeros(cap, dtype=np.int32)
    dist = np.zeros(cap)
    val = np.zeros(cap)
    out.capacity = cap
    out.point = N.as_ptr(point, C.c_int64)
    out.atom = N.as_ptr(atom, C.c_int32)
    out.distance = N.as_ptr(dist, C.c_double)
    out.value = N.as_ptr(val, C.c_double)
    N.raise_for(lib.cm_grid3d(C.byref(desc), C.byref(out)), None)
    k = int(out.count)
    return point[:k], atom[:k], dist[:k], val[:k], tuple(int(v) for v in out.n), np.array(list(out.origin))
