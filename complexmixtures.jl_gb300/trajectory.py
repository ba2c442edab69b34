"""Trajectory plugin interface and readers (src/Trajectory.jl:11-249,
src/trajectory_formats/NamdDCD.jl, src/trajectory_formats/PDBTraj.jl).

A trajectory exposes the reference's plugin methods -- ``opentraj``,
``firstframe``, ``nextframe``, ``getunitcell``, ``closetraj`` -- and the
fields ``nframes``, ``solute``, ``solvent``, ``x_solute``, ``x_solvent``
(coordinates of the current frame, selection order).  Unit cells are 3x3
matrices whose columns are the lattice vectors.
"""
from __future__ import annotations

import math
import os
import struct
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from .options import Options
from .selection import AtomSelection


class Trajectory:
    """Base class of the trajectory plugins (src/Trajectory.jl:11)."""

    filename: str = ""
    nframes: int = 0
    solute: AtomSelection
    solvent: AtomSelection
    x_solute: np.ndarray
    x_solvent: np.ndarray

    def opentraj(self):
        raise NotImplementedError

    def firstframe(self):
        raise NotImplementedError

    def nextframe(self):
        raise NotImplementedError

    def getunitcell(self) -> np.ndarray:
        raise NotImplementedError

    def closetraj(self):
        raise NotImplementedError

    # the reference's `lastatom` / coordinate gather, shared by file readers
    def _gather(self, xyz: np.ndarray):
        s = np.asarray(self.solute.indices, dtype=np.int64) - 1
        v = np.asarray(self.solvent.indices, dtype=np.int64) - 1
        self.x_solute = xyz[s].astype(np.float64)
        self.x_solvent = xyz[v].astype(np.float64)


class ArrayTrajectory(Trajectory):
    """Frames already in memory: ``frames`` [nframes, natoms, 3] (all atoms of
    the system, indexed by the selections' 1-based indices) or the pre-gathered
    ``solute_frames`` / ``solvent_frames`` arrays; ``cells`` [nframes, 3, 3]."""

    def __init__(self, solute: AtomSelection, solvent: Optional[AtomSelection] = None, *, frames=None,
                 solute_frames=None, solvent_frames=None, cells=None, filename: str = "<memory>"):
        self.solute = solute
        self.solvent = solvent if solvent is not None else solute
        self.filename = filename
        if frames is not None:
            frames = np.asarray(frames)
            s = np.asarray(self.solute.indices, dtype=np.int64) - 1
            v = np.asarray(self.solvent.indices, dtype=np.int64) - 1
            self._xs = frames[:, s]
            self._xv = frames[:, v]
        else:
            self._xs = np.asarray(solute_frames)
            self._xv = np.asarray(solvent_frames) if solvent_frames is not None else self._xs
        self.nframes = int(self._xs.shape[0])
        self._cells = np.asarray(cells, dtype=np.float64).reshape(self.nframes, 3, 3)
        self._i = -1
        self.x_solute = np.zeros((self.solute.natoms(), 3))
        self.x_solvent = np.zeros((self.solvent.natoms(), 3))

    def opentraj(self):
        self._i = -1

    def firstframe(self):
        self._i = -1

    def nextframe(self):
        self._i += 1
        self.x_solute = self._xs[self._i]
        self.x_solvent = self._xv[self._i]

    def getunitcell(self):
        return self._cells[max(self._i, 0)]

    def closetraj(self):
        pass

    # bulk access used by the driver to hand many frames to the GPU at once
    def frame_arrays(self, idx: Sequence[int]):
        idx = np.asarray(idx, dtype=np.int64)
        return self._xs[idx], self._xv[idx], self._cells[idx]


def unitcell_from_lengths_angles(a: float, b: float, c: float, alpha: float, beta: float, gamma: float) -> np.ndarray:
    """Cell matrix (columns = lattice vectors) from lengths and angles in
    degrees, in the orientation of Chemfiles' UnitCell (a along x, b in the xy
    plane) that the reference transposes into its column convention
    (src/trajectory_formats/NamdDCD.jl:175-188).  Right angles give a diagonal
    matrix."""
    if alpha == 90.0 and beta == 90.0 and gamma == 90.0:
        return np.diag([a, b, c]).astype(np.float64)
    ca, cb, cg = (math.cos(math.radians(x)) for x in (alpha, beta, gamma))
    sg = math.sin(math.radians(gamma))
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz = math.sqrt(max(c * c - cx * cx - cy * cy, 0.0))
    return np.array([[a, b * cg, cx], [0.0, b * sg, cy], [0.0, 0.0, cz]], dtype=np.float64)


class NamdDCD(Trajectory):
    """NAMD DCD reader (src/trajectory_formats/NamdDCD.jl:16-229): Fortran
    unformatted records, float32 x/y/z blocks, six doubles of unit cell per
    frame (A, gamma, B, beta, alpha, C; zero angles mean 90 degrees)."""

    def __init__(self, filename: str, solute: AtomSelection, solvent: Optional[AtomSelection] = None, lastframe: int = -1):
        self.filename = filename
        self.solute = solute
        self.solvent = solvent if solvent is not None else solute
        with open(filename, "rb") as f:
            self._endian = self._detect(f)
            hdr = self._record(f)
            if len(hdr) < 84 or hdr[:4] != b"CORD":
                raise ValueError(f"{filename}: not a DCD file")
            self._record(f)  # title
            (self.natoms_file,) = struct.unpack(self._endian + "i", self._record(f))
            self._data_start = f.tell()
            first = self._record(f)
            if len(first) != 48:
                raise ValueError("DCD file does not contain unit cell information.")
        self.lastatom = max(max(solute.indices), max(self.solvent.indices))
        if self.lastatom > self.natoms_file:
            raise ValueError("selection indices beyond the number of atoms in the DCD file")
        frame_bytes = (8 + 48) + 3 * (8 + 4 * self.natoms_file)
        size = os.path.getsize(filename)
        n = (size - self._data_start) // frame_bytes
        self.nframes = int(n if lastframe < 0 else min(n, lastframe))
        self._f = None
        self._unitcell = np.zeros(6)
        self.x_solute = np.zeros((solute.natoms(), 3))
        self.x_solvent = np.zeros((self.solvent.natoms(), 3))

    @staticmethod
    def _detect(f) -> str:
        raw = f.read(4)
        f.seek(0)
        return "<" if struct.unpack("<i", raw)[0] == 84 else ">"

    def _record(self, f) -> bytes:
        (n,) = struct.unpack(self._endian + "i", f.read(4))
        data = f.read(n)
        (m,) = struct.unpack(self._endian + "i", f.read(4))
        if m != n or len(data) != n:
            raise ValueError("corrupted Fortran record in DCD file")
        return data

    def opentraj(self):
        self._f = open(self.filename, "rb")
        self.firstframe()

    def firstframe(self):
        self._f.seek(self._data_start)

    def nextframe(self):
        f = self._f
        self._unitcell = np.frombuffer(self._record(f), dtype=self._endian + "f8").copy()
        x = np.frombuffer(self._record(f), dtype=self._endian + "f4")
        y = np.frombuffer(self._record(f), dtype=self._endian + "f4")
        z = np.frombuffer(self._record(f), dtype=self._endian + "f4")
        self._gather(np.stack([x, y, z], axis=1))

    def getunitcell(self):
        return self._cell_of(self._unitcell)

    @staticmethod
    def _cell_of(uc):
        A, gamma, B, beta, alpha, Cc = (float(x) for x in uc)
        if alpha == 0.0 or beta == 0.0 or gamma == 0.0:
            alpha = beta = gamma = 90.0
        return unitcell_from_lengths_angles(A, B, Cc, alpha, beta, gamma)

    # raw frames for the engine's device-side decode (cm_set_dcd_layout)
    @property
    def frame_bytes(self) -> int:
        return (8 + 48) + 3 * (8 + 4 * self.natoms_file)

    def dcd_layout(self) -> dict:
        """Byte layout of one frame: the unit-cell record, then the x, y and
        z records (each float32 array behind a 4-byte marker)."""
        n4 = 4 * self.natoms_file
        x = 56 + 4
        return dict(natoms=self.natoms_file, frame_bytes=self.frame_bytes, x_offset=x, y_offset=x + n4 + 8,
                    z_offset=x + 2 * (n4 + 8), big_endian=self._endian == ">")

    def read_raw(self, first: int, n: int):
        """Frames first .. first + n - 1 (0-based) as bytes [n, frame_bytes]
        and their cells [n, 3, 3]; the record markers are checked."""
        fb = self.frame_bytes
        with open(self.filename, "rb") as f:
            f.seek(self._data_start + first * fb)
            raw = np.fromfile(f, dtype=np.uint8, count=n * fb)
        if raw.size != n * fb:
            raise ValueError("DCD file ends inside a frame")
        raw = raw.reshape(n, fb)
        marks = raw.view(self._endian + "i4")
        n4 = 4 * self.natoms_file
        want = {0: 48, 13: 48}
        for k in range(3):
            o = 56 + k * (n4 + 8)
            want[o // 4] = n4
            want[(o + 4 + n4) // 4] = n4
        for col, val in want.items():
            if np.any(marks[:, col] != val):
                raise ValueError("corrupted Fortran record in DCD file")
        uc = np.ascontiguousarray(raw[:, 4:52]).view(self._endian + "f8").reshape(n, 6)
        cells = np.stack([self._cell_of(u) for u in uc])
        return raw, cells

    def closetraj(self):
        if self._f:
            self._f.close()
            self._f = None


class PDBTraj(Trajectory):
    """Multi-model PDB trajectory (src/trajectory_formats/PDBTraj.jl): frames
    separated by END / ENDMDL, unit cell from each frame's CRYST1 record; atom
    indices are positions in the frame (1-based)."""

    def __init__(self, filename: str, solute: AtomSelection, solvent: Optional[AtomSelection] = None):
        self.filename = filename
        self.solute = solute
        self.solvent = solvent if solvent is not None else solute
        self._frames, self._cells = self._parse(filename)
        self.nframes = len(self._frames)
        self._i = -1
        self.x_solute = np.zeros((solute.natoms(), 3))
        self.x_solvent = np.zeros((self.solvent.natoms(), 3))

    @staticmethod
    def _parse(filename):
        frames, cells = [], []
        cur, cell = [], None
        with open(filename) as f:
            for line in f:
                rec = line[:6]
                if rec.startswith("CRYST1"):
                    # whitespace-separated: some writers do not keep the PDB columns
                    t = line.split()
                    a, b, c = float(t[1]), float(t[2]), float(t[3])
                    al, be, ga = float(t[4]), float(t[5]), float(t[6])
                    cell = unitcell_from_lengths_angles(a, b, c, al, be, ga)
                elif rec.startswith("ATOM") or rec.startswith("HETATM"):
                    cur.append((float(line[30:38]), float(line[38:46]), float(line[46:54])))
                elif rec.startswith("END"):
                    if cur:
                        frames.append(np.array(cur))
                        cells.append(cell)
                    cur = []
        if cur:
            frames.append(np.array(cur))
            cells.append(cell)
        return frames, cells

    def opentraj(self):
        self._i = -1

    def firstframe(self):
        self._i = -1

    def nextframe(self):
        self._i += 1
        self._gather(self._frames[self._i])

    def getunitcell(self):
        return self._cells[max(self._i, 0)]

    def closetraj(self):
        pass


def make_trajectory(filename: str, solute: AtomSelection, solvent: Optional[AtomSelection] = None, *,
                    format: str = "", lastframe: int = -1) -> Trajectory:
    """Format dispatch of Trajectory(filename, solute, solvent; format)
    (src/Trajectory.jl:31-63): DCD and PDB are read natively; other formats
    (Chemfiles) are outside the engine."""
    ext = filename.rsplit(".", 1)[-1].lower() if "." in filename else ""
    if format and format not in ("dcd", "PDBTraj"):
        raise ValueError(f"Trajectory format not properly set: {format}. Available trajectory formats: dcd, PDBTraj")
    if format == "dcd" or (not format and ext == "dcd"):
        return NamdDCD(filename, solute, solvent, lastframe=lastframe)
    if format == "PDBTraj" or (not format and ext == "pdb"):
        return PDBTraj(filename, solute, solvent)
    raise ValueError(f"unsupported trajectory format for {filename}")


def convert_unitcell(unitcell, tol: float = 1e-10):
    """Diagonal (relative tol) cells become length-3 vectors, others stay 3x3
    (src/Trajectory.jl:72-77)."""
    m = np.asarray(unitcell, dtype=np.float64)
    if m.shape != (3, 3):
        raise ValueError("Unit cell must be a 3x3 matrix.")
    s = abs(min(np.diag(m)))
    off = [abs(m[i, j]) for i in range(3) for j in range(3) if i != j]
    if all(o < tol * s for o in off):
        return np.diag(m).copy()
    return m.copy()


def cell_matrix(unitcell) -> np.ndarray:
    """3x3 matrix of a cell given as a 3-vector (orthorhombic) or a matrix."""
    u = np.asarray(unitcell, dtype=np.float64)
    return np.diag(u) if u.shape == (3,) else u


@dataclass
class TrajectoryMetaData:
    """src/Trajectory.jl:180-187."""

    irefatom: int
    lastframe_read: int
    nframes_read: int
    n_groups_solute: int
    n_groups_solvent: int
    unitcell: np.ndarray


def trajectory_metadata(trajectory: Trajectory, options: Options) -> TrajectoryMetaData:
    """src/Trajectory.jl:189-249, including the default reference atom: the atom
    of the first solvent molecule closest to that molecule's mean position in
    the first frame (first index on ties)."""
    if options.irefatom > trajectory.solvent.natomspermol:
        raise ValueError(
            f"in MDDF options: Reference atom index {options.irefatom} is greater than number of atoms of the "
            "solvent molecule. "
        )
    if options.lastframe > trajectory.nframes:
        raise ValueError("in MDDF options: lastframe is greater than trajectory.nframes. ")
    trajectory.opentraj()
    trajectory.firstframe()
    trajectory.nextframe()
    unitcell = convert_unitcell(trajectory.getunitcell())
    if options.irefatom == -1:
        mol = np.asarray(trajectory.x_solvent[: trajectory.solvent.natomspermol], dtype=np.float64)
        cm = mol.mean(axis=0)
        dist = np.sqrt(((mol - cm) ** 2).sum(axis=1))
        irefatom = int(np.argmin(dist)) + 1
    else:
        irefatom = options.irefatom
    lastframe_read = trajectory.nframes if options.lastframe == -1 else options.lastframe
    nframes_read = len(range(options.firstframe, lastframe_read + 1, options.stride))
    trajectory.closetraj()
    return TrajectoryMetaData(
        irefatom=irefatom,
        lastframe_read=lastframe_read,
        nframes_read=nframes_read,
        n_groups_solute=trajectory.solute.ngroups(),
        n_groups_solvent=trajectory.solvent.ngroups(),
        unitcell=unitcell,
    )
