"""Engine: one GPU handle of libcmgpu.so for one (solute, solvent, options) system.

This is the step the reference performs per frame with ``mddf_frame!`` /
``coordination_number_frame!`` (src/mddf.jl:361-471) and per chunk with
``sum!`` (src/results.jl:629-649): frames go in, frame-weighted histogram
counts come out.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _native as N

_PRECISION = {"fp64": N.CM_PRECISION_FP64, "fp32": N.CM_PRECISION_FP32_GUARD}
_REGIME = {"auto": N.CM_REGIME_AUTO, "pairs": N.CM_REGIME_PAIRS, "atoms": N.CM_REGIME_ATOMS}


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


SCHEDULES = {"auto": N.CM_SCHED_AUTO, "cell": N.CM_SCHED_CELL, "balanced": N.CM_SCHED_BALANCED}
SCHEDULE_NAMES = {v: k for k, v in SCHEDULES.items()}
REAL_PASSES = {"auto": N.CM_REAL_AUTO, "warp": N.CM_REAL_WARP, "tile": N.CM_REAL_TILE}
REAL_PASS_NAMES = {v: k for k, v in REAL_PASSES.items()}


def system_desc(
    *,
    solute_nmols: int,
    solute_natomspermol: int,
    solvent_nmols: int,
    solvent_natomspermol: int,
    autocorrelation: bool,
    irefatom: int,
    cutoff: float,
    binstep: float,
    dbulk: float,
    usecutoff: bool,
    nbins: int,
    n_random_samples: int,
    lcell: int = 1,
    coordination_number_only: bool = False,
    precision: str = "fp32",
    regime: str = "auto",
    seed: int = 321,
    solute_groups: Optional[Sequence[Sequence[int]]] = None,
    solute_ngroups: int = 0,
    solvent_groups: Optional[Sequence[Sequence[int]]] = None,
    solvent_ngroups: int = 0,
    device: int = 0,
    max_frames_per_batch: int = 0,
    hbm_budget_bytes: int = 0,
    kernel_timing: bool = False,
    cell_scale_pct: int = 0,
    launch: str = "auto",
    atoms_schedule: str = "auto",
    guard_queue_capacity: int = 0,
    real_pass: str = "auto",
    atoms_grid: int = 0,
    atoms_grid_capacity: int = 0,
):
    """cm_system_desc of a system, and the arrays it points to (keep them
    alive while the description is in use).  ``cell_scale_pct`` scales the
    search cells (speed only; see ``autotune``); ``launch`` ("auto", "stream"
    or "graph") says whether each compute chunk's kernels are launched one by
    one or replayed as a captured CUDA graph; ``atoms_schedule`` ("auto",
    "cell" or "balanced") picks the ATOMS-layout evaluation schedule (both
    speed only); ``guard_queue_capacity`` (0 = sized by the engine) bounds the
    FP32 real pass's guard and edge queues per compute chunk: a chunk that
    overflows them is redone on the device without queues, so the counts do
    not depend on it; ``real_pass`` ("auto", "warp" or "tile") picks the FP32
    real-pass schedule of the molecule layout (speed only); ``atoms_grid``
    (ATOMS layout, one solute molecule, FP32) sets the fine cells per
    search-cell axis of the per-frame candidate grid (1-6; 0 = fine cells of
    about 2.5 A for dense solutes, the walk for sparse ones; -1 = no grid,
    every query walks the stencil; speed only) and
    ``atoms_grid_capacity`` its list entries per frame (0 = sized by the
    engine; a frame whose lists do not fit walks the stencil)."""
    d = N.cm_system_desc()
    d.api_version = N.CM_API_VERSION
    d.solute_nmols = solute_nmols
    d.solute_natomspermol = solute_natomspermol
    d.solvent_nmols = solvent_nmols
    d.solvent_natomspermol = solvent_natomspermol
    d.autocorrelation = 1 if autocorrelation else 0
    d.irefatom = irefatom
    d.cutoff = cutoff
    d.binstep = binstep
    d.dbulk = dbulk
    d.usecutoff = 1 if usecutoff else 0
    d.nbins = nbins
    d.n_random_samples = n_random_samples
    d.lcell = lcell
    d.mode = N.CM_MODE_COORDINATION_NUMBER if coordination_number_only else N.CM_MODE_MDDF
    d.precision = _PRECISION[precision]
    d.regime = _REGIME[regime]
    d.seed = seed & 0xFFFFFFFFFFFFFFFF
    keep = []
    if solute_groups is not None:
        off, idx = N.csr(solute_groups, solute_natomspermol)
        keep += [off, idx]
        d.solute_ngroups = solute_ngroups
        d.solute_group_offsets = N.as_ptr(off, C.c_int64)
        d.solute_groups = N.as_ptr(idx, C.c_int32)
    if solvent_groups is not None:
        off, idx = N.csr(solvent_groups, solvent_nmols * solvent_natomspermol)
        keep += [off, idx]
        d.solvent_ngroups = solvent_ngroups
        d.solvent_group_offsets = N.as_ptr(off, C.c_int64)
        d.solvent_groups = N.as_ptr(idx, C.c_int32)
    d.device = device
    d.max_frames_per_batch = max_frames_per_batch
    d.hbm_budget_bytes = hbm_budget_bytes
    d.kernel_timing = 1 if kernel_timing else 0
    d.cell_scale_pct = cell_scale_pct
    modes = {"auto": N.CM_LAUNCH_AUTO, "stream": N.CM_LAUNCH_STREAM, "graph": N.CM_LAUNCH_GRAPH}
    if launch not in modes:
        raise ValueError(f"launch must be one of {sorted(modes)}")
    d.launch = modes[launch]
    if atoms_schedule not in SCHEDULES:
        raise ValueError(f"atoms_schedule must be one of {sorted(SCHEDULES)}")
    d.atoms_schedule = SCHEDULES[atoms_schedule]
    d.guard_queue_capacity = guard_queue_capacity
    if real_pass not in REAL_PASSES:
        raise ValueError(f"real_pass must be one of {sorted(REAL_PASSES)}")
    d.real_pass = REAL_PASSES[real_pass]
    if not -1 <= int(atoms_grid) <= 6:
        raise ValueError("atoms_grid must be -1, 0 or 1-6")
    d.atoms_grid = int(atoms_grid)
    if atoms_grid_capacity < 0:
        raise ValueError("atoms_grid_capacity must be >= 0")
    d.atoms_grid_capacity = int(atoms_grid_capacity)
    return d, keep


def autotune(solute_xyz, solvent_xyz, cells, frame_ids=None, **system) -> dict:
    """Time the candidate search-cell sizes, and with each the evaluation
    schedules (ATOMS layout: cell and balanced; self-MDDF in the molecule
    layout: home-cell tiles and warps per molecule), on sample frames
    (cm_autotune); a single solute molecule in the ATOMS layout (FP32) also
    tries the candidate grid at several fine-cell counts (atoms_grid=-1 keeps
    it out).
    Returns the fastest as {"cell_scale_pct", "atoms_schedule", "real_pass",
    "atoms_grid"} plus "candidates", a list of the same keys with
    "ms_per_frame"; pass the first four to Engine."""
    lib = N.load()
    system = {k: v for k, v in system.items()
              if k not in ("cell_scale_pct", "atoms_schedule", "real_pass") and not (k == "atoms_grid" and v >= 0)}
    d, keep = system_desc(**system)
    Ns = d.solute_nmols * d.solute_natomspermol
    Nv = d.solvent_nmols * d.solvent_natomspermol
    fr, keep_f = frames_struct(solute_xyz, solvent_xyz, cells, None, frame_ids, Ns, Nv, bool(d.autocorrelation))
    t = N.cm_tuning()
    N.raise_for(lib.cm_autotune(C.byref(d), C.byref(fr), C.byref(t)), None)
    del keep, keep_f
    atoms = d.regime == N.CM_REGIME_ATOMS or (d.regime == N.CM_REGIME_AUTO and max(
        d.solute_natomspermol, d.solvent_natomspermol) > 32)
    out = {"cell_scale_pct": t.cell_scale_pct, "atoms_schedule": SCHEDULE_NAMES[t.atoms_schedule],
           "real_pass": REAL_PASS_NAMES[t.real_pass], "atoms_grid": t.atoms_grid, "candidates": []}
    for i in range(t.ncandidates):
        c = {"cell_scale_pct": t.candidates[i], "ms_per_frame": t.ms_per_frame[i], "atoms_grid": t.grids[i]}
        if atoms:
            c["atoms_schedule"] = SCHEDULE_NAMES[t.schedules[i]]
        else:
            c["atoms_schedule"] = "auto"
            c["real_pass"] = REAL_PASS_NAMES[t.schedules[i]]
        out["candidates"].append(c)
    return out


def memory_cache(device: int = 0, release: bool = False) -> dict:
    """Free device and pinned host bytes held by the process-wide block cache
    that closed engines return their memory to (cm_memory_cache); with
    ``release`` they are first handed back to the driver."""
    lib = N.load()
    dev, host = C.c_int64(0), C.c_int64(0)
    N.raise_for(lib.cm_memory_cache(int(device), 1 if release else 0, C.byref(dev), C.byref(host)), None)
    return {"device_bytes": dev.value, "host_bytes": host.value}


def frames_struct(solute_xyz, solvent_xyz, cells, weights, frame_ids, natoms_solute, natoms_solvent, autocorrelation):
    """cm_frames for a batch of frames, and the arrays it points to.  Frames
    that are slices of a larger array (each frame's atoms contiguous, the
    frames further apart) are passed with their frame stride, not copied."""
    xs, kind_s, mem_s, ss = _coords(solute_xyz, natoms_solute)
    nf = int(xs.shape[0])
    xv, vs = None, 0
    if not autocorrelation:
        xv, kind_v, mem_v, vs = _coords(solvent_xyz, natoms_solvent)
        if kind_v != kind_s or mem_v != mem_s:
            raise ValueError("solute and solvent coordinates must share dtype and device")
    cells = np.asarray(cells, dtype=np.float64).reshape(nf, 3, 3)
    # column-major 3x3 (columns are lattice vectors) == C-order transpose
    cm = np.ascontiguousarray(np.transpose(cells, (0, 2, 1))).reshape(nf, 9)
    w = None if weights is None else np.ascontiguousarray(np.asarray(weights, dtype=np.float64).reshape(nf))
    ids = np.arange(1, nf + 1, dtype=np.int64) if frame_ids is None else np.ascontiguousarray(
        np.asarray(frame_ids, dtype=np.int64).reshape(nf))
    fr = N.cm_frames()
    fr.nframes = nf
    fr.coord_type = kind_s
    fr.memory = mem_s
    fr.solute_xyz = _ptr(xs)
    fr.solvent_xyz = _ptr(xv) if xv is not None else None
    fr.cells = N.as_ptr(cm, C.c_double)
    fr.weights = N.as_ptr(w, C.c_double) if w is not None else None
    fr.frame_ids = N.as_ptr(ids, C.c_int64)
    fr.solute_frame_stride = ss
    fr.solvent_frame_stride = vs
    return fr, [xs, xv, cm, w, ids]


def _ptr(x):
    if x is None:
        return None
    if _is_torch(x):
        return C.c_void_p(x.data_ptr())
    return C.c_void_p(x.ctypes.data)


def _frame_stride(shape, strides, natoms):
    """Element stride between frames when each frame's [natoms, 3] block is
    contiguous (0 when the frames are consecutive too), else None."""
    if strides[2] != 1 or (natoms > 1 and strides[1] != 3):
        return None
    if shape[0] == 1 or strides[0] == natoms * 3:
        return 0
    return strides[0] if strides[0] >= natoms * 3 else None


def _coords(x, natoms):
    if _is_torch(x):
        import torch

        if x.dtype not in (torch.float32, torch.float64):
            raise ValueError("coordinates must be float32 or float64")
        if x.dim() == 2:
            x = x.unsqueeze(0)
        if x.shape[1] != natoms or x.shape[2] != 3:
            raise ValueError(f"coordinates must be [nframes, {natoms}, 3]")
        stride = _frame_stride(tuple(x.shape), tuple(x.stride()), natoms)
        if stride is None:
            x, stride = x.contiguous(), 0
        kind = N.CM_COORD_F32 if x.dtype == torch.float32 else N.CM_COORD_F64
        mem = N.CM_MEM_DEVICE if x.is_cuda else N.CM_MEM_HOST
        return x, kind, mem, stride
    a = np.asarray(x)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    if a.ndim == 2:
        a = a[None]
    if a.shape[1] != natoms or a.shape[2] != 3:
        raise ValueError(f"coordinates must be [nframes, {natoms}, 3]")
    stride = None
    if all(v % a.itemsize == 0 for v in a.strides):
        stride = _frame_stride(a.shape, tuple(v // a.itemsize for v in a.strides), natoms)
    if stride is None:
        a, stride = np.ascontiguousarray(a), 0
    return a, (N.CM_COORD_F32 if a.dtype == np.float32 else N.CM_COORD_F64), N.CM_MEM_HOST, stride


def counts_arrays(nbins, ngroups_solute, ngroups_solvent):
    """Zeroed output arrays of cm_read_counts and the struct pointing to them."""
    out = {
        "md_count": np.zeros(nbins),
        "md_count_random": np.zeros(nbins),
        "rdf_count": np.zeros(nbins),
        "rdf_count_random": np.zeros(nbins),
        "solute_group_count": np.zeros((ngroups_solute, nbins)),
        "solute_group_count_random": np.zeros((ngroups_solute, nbins)),
        "solvent_group_count": np.zeros((ngroups_solvent, nbins)),
        "solvent_group_count_random": np.zeros((ngroups_solvent, nbins)),
    }
    c = N.cm_counts()
    for k, v in out.items():
        setattr(c, k, N.as_ptr(v, C.c_double))
    return out, c


def raw_arrays(nbins, ngroups_solute, ngroups_solvent):
    """Zeroed output arrays of cm_read_raw_counts and the struct pointing to them."""
    out = {
        "md": np.zeros(nbins, np.int64),
        "md_random": np.zeros(nbins, np.int64),
        "rdf": np.zeros(nbins, np.int64),
        "rdf_random": np.zeros(nbins, np.int64),
        "solute_group": np.zeros((ngroups_solute, nbins), np.int64),
        "solute_group_random": np.zeros((ngroups_solute, nbins), np.int64),
        "solvent_group": np.zeros((ngroups_solvent, nbins), np.int64),
        "solvent_group_random": np.zeros((ngroups_solvent, nbins), np.int64),
    }
    c = N.cm_raw_counts()
    for k, v in out.items():
        setattr(c, k, N.as_ptr(v, C.c_int64))
    return out, c


class Engine:
    """GPU engine handle.

    Parameters follow the reference's Options / AtomSelection / Result fields
    (see ``system_desc``).  ``solute_groups`` is a list, per atom of one solute
    molecule (local index), of the group numbers it credits; ``solvent_groups``
    the same per atom of the whole solvent selection.  ``None`` means default
    per-atom-type groups.
    """

    def __init__(self, **kw):
        self._lib = N.load()
        self._h = C.c_void_p()
        d, self._keep = system_desc(**kw)
        st = self._lib.cm_create(C.byref(d), C.byref(self._h))
        N.raise_for(st, None)
        self.desc = d
        self.nbins = d.nbins
        self.ngroups_solute = d.solute_ngroups if kw.get("solute_groups") is not None else d.solute_natomspermol
        self.ngroups_solvent = d.solvent_ngroups if kw.get("solvent_groups") is not None else d.solvent_natomspermol
        self.autocorrelation = bool(d.autocorrelation)
        self.Ns = d.solute_nmols * d.solute_natomspermol
        self.Nv = d.solvent_nmols * d.solvent_natomspermol
        self._inflight = []

    # -------------------------------------------------------------- frames
    def submit(self, solute_xyz, solvent_xyz, cells, weights=None, frame_ids=None) -> None:
        """Add frames.  Coordinates are [nframes, natoms, 3] float32/float64
        numpy arrays (host) or torch tensors (host or CUDA); cells are
        [nframes, 3, 3] matrices whose columns are the lattice vectors."""
        fr, keep = frames_struct(solute_xyz, solvent_xyz, cells, weights, frame_ids, self.Ns, self.Nv,
                                 self.autocorrelation)
        st = self._lib.cm_submit_frames(self._h, C.byref(fr))
        N.raise_for(st, self._h)
        # device and pinned inputs are read asynchronously: hold them (and any
        # contiguous copies made here) until the next synchronising call
        self._inflight.append(keep)

    def set_dcd_layout(self, *, natoms, frame_bytes, x_offset, y_offset, z_offset, big_endian, solute_atoms,
                       solvent_atoms=None) -> None:
        """Declare the raw DCD frame layout and the selections' 0-based atom
        indices in the frame (cm_set_dcd_layout), for ``submit_dcd``."""
        s = np.ascontiguousarray(np.asarray(solute_atoms, dtype=np.int32).reshape(-1))
        v = None if solvent_atoms is None else np.ascontiguousarray(np.asarray(solvent_atoms, dtype=np.int32).reshape(-1))
        if s.size != self.Ns or (v is not None and v.size != self.Nv):
            raise ValueError("one atom index per selection atom")
        L = N.cm_dcd_layout(natoms=natoms, frame_bytes=frame_bytes, x_offset=x_offset, y_offset=y_offset,
                            z_offset=z_offset, big_endian=1 if big_endian else 0)
        L.solute_atoms = N.as_ptr(s, C.c_int32)
        L.solvent_atoms = N.as_ptr(v, C.c_int32) if v is not None else None
        N.raise_for(self._lib.cm_set_dcd_layout(self._h, C.byref(L)), self._h)

    def submit_dcd(self, raw, cells, weights=None, frame_ids=None) -> None:
        """Add frames given as raw DCD bytes [nframes, frame_bytes] (uint8
        numpy array, or torch tensor on the host or the device); the engine
        gathers the selections on the device."""
        if _is_torch(raw):
            nf = int(raw.shape[0])
            keep_raw = raw.contiguous()
            mem = N.CM_MEM_DEVICE if keep_raw.is_cuda else N.CM_MEM_HOST
            ptr = keep_raw.data_ptr()
        else:
            keep_raw = np.ascontiguousarray(np.asarray(raw, dtype=np.uint8))
            nf = int(keep_raw.shape[0])
            mem = N.CM_MEM_HOST
            ptr = keep_raw.ctypes.data
        cells = np.asarray(cells, dtype=np.float64).reshape(nf, 3, 3)
        cm = np.ascontiguousarray(np.transpose(cells, (0, 2, 1))).reshape(nf, 9)
        w = None if weights is None else np.ascontiguousarray(np.asarray(weights, dtype=np.float64).reshape(nf))
        ids = np.arange(1, nf + 1, dtype=np.int64) if frame_ids is None else np.ascontiguousarray(
            np.asarray(frame_ids, dtype=np.int64).reshape(nf))
        fr = N.cm_frames()
        fr.nframes = nf
        fr.coord_type = N.CM_COORD_DCD
        fr.memory = mem
        fr.solute_xyz = C.c_void_p(ptr)
        fr.solvent_xyz = None
        fr.cells = N.as_ptr(cm, C.c_double)
        fr.weights = N.as_ptr(w, C.c_double) if w is not None else None
        fr.frame_ids = N.as_ptr(ids, C.c_int64)
        N.raise_for(self._lib.cm_submit_frames(self._h, C.byref(fr)), self._h)
        self._inflight.append([keep_raw, cm, w, ids])

    # -------------------------------------------------------------- output
    def counts(self) -> dict:
        """Frame-weighted counts (the Result fields before finalresults!)."""
        out, c = counts_arrays(self.nbins, self.ngroups_solute, self.ngroups_solvent)
        st = self._lib.cm_read_counts(self._h, C.byref(c))
        N.raise_for(st, self._h)
        self._inflight.clear()
        out["volume_total"] = c.volume_total
        out["weight_total"] = c.weight_total
        out["frames"] = c.frames
        return out

    def results(self, frame_weight_sum: float = 0.0) -> dict:
        """Finalised Result fields computed on the device (cm_read_results):
        the vectors of finalresults! plus volumes, densities, density_fix
        and the count of random bins without samples."""
        nb = self.nbins
        gv = self.ngroups_solute if self.autocorrelation else self.ngroups_solvent
        out = {k: np.zeros(nb) for k in N.RESULT_VECTORS}
        out.update({k: np.zeros((self.ngroups_solute if k.startswith("solute") else gv, nb)) for k in N.RESULT_GROUPS})
        r = N.cm_results()
        for k in N.RESULT_VECTORS + N.RESULT_GROUPS:
            setattr(r, k, N.as_ptr(out[k], C.c_double))
        st = self._lib.cm_read_results(self._h, float(frame_weight_sum), C.byref(r))
        N.raise_for(st, self._h)
        self._inflight.clear()
        for k in N.RESULT_SCALARS:
            out[k] = getattr(r, k)
        out["zero_random_bins"] = r.zero_random_bins
        return out

    def contributions(self, queries, frame_weight_sum: float = 0.0) -> np.ndarray:
        """Group contributions on the device (cm_contributions), one row per
        query.  A query is (side, type, rows, divide): side "solute" or
        "solvent", type "mddf" / "coordination_number" / "md_count" / "kbi",
        the 0-based group rows summed in order, and whether each row is divided
        by the side's nmols.  ``contribution_terms`` resolves a SoluteGroup or
        SolventGroup into (side, rows, divide)."""
        nq = len(queries)
        if nq == 0:
            return np.zeros((0, self.nbins))
        arr = (N.cm_contrib_query * nq)()
        keep = []
        for k, (side, type, rows, divide) in enumerate(queries):
            if side not in ("solute", "solvent"):
                raise ValueError("side must be 'solute' or 'solvent'")
            if type not in N.CM_CONTRIB_TYPES:
                raise ValueError("type must be :mddf (default), :coordination_number, :md_count, :kbi")
            g = np.ascontiguousarray(rows, dtype=np.int32)
            keep.append(g)
            arr[k].side = N.CM_GROUP_SOLUTE if side == "solute" else N.CM_GROUP_SOLVENT
            arr[k].type = N.CM_CONTRIB_TYPES[type]
            arr[k].divide = 1 if divide else 0
            arr[k].nterms = len(g)
            arr[k].groups = N.as_ptr(g, C.c_int32)
        out = np.zeros((nq, self.nbins))
        st = self._lib.cm_contributions(self._h, float(frame_weight_sum), nq, arr, N.as_ptr(out, C.c_double))
        N.raise_for(st, self._h)
        self._inflight.clear()
        return out

    def raw_counts(self) -> dict:
        """Exact int64 half-unit counts (runs with a single frame weight)."""
        out, c = raw_arrays(self.nbins, self.ngroups_solute, self.ngroups_solvent)
        st = self._lib.cm_read_raw_counts(self._h, C.byref(c))
        N.raise_for(st, self._h)
        self._inflight.clear()
        return out

    def snapshot(self) -> dict:
        """Exact state of the accumulators for a later resume: the half-unit
        counts, the frame weight they were computed with, the frames and the
        weighted volume sum (single-weight runs, as ``raw_counts``)."""
        snap = self.raw_counts()
        w = C.c_double(0.0)
        N.raise_for(self._lib.cm_raw_counts_weight(self._h, C.byref(w)), self._h)
        c = self.counts()
        snap.update(frame_weight=w.value, frames=int(c["frames"]), volume_total=float(c["volume_total"]))
        return snap

    def restore(self, snap: dict) -> None:
        """Load a snapshot (``snapshot``, ``load_snapshot`` or
        ``snapshot_from_result``) into this engine (cm_load_raw_counts):
        frames submitted afterwards add to it, so frames 1..k, a snapshot and
        frames k+1..n on a restored engine give the counts of one run over
        1..n."""
        keep = {}
        c = N.cm_raw_counts()
        for k in ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
                  "solvent_group_random"):
            if k.startswith("solvent") and self.autocorrelation:
                continue
            keep[k] = np.ascontiguousarray(snap[k], dtype=np.int64)
            setattr(c, k, N.as_ptr(keep[k], C.c_int64))
        st = self._lib.cm_load_raw_counts(self._h, C.byref(c), float(snap["frame_weight"]), int(snap["frames"]),
                                          float(snap["volume_total"]))
        N.raise_for(st, self._h)

    def stats(self) -> dict:
        s = N.cm_stats()
        st = self._lib.cm_get_stats(self._h, C.byref(s))
        N.raise_for(st, self._h)
        return {name: getattr(s, name) for name, _ in N.cm_stats._fields_}

    def kernel_times(self) -> dict:
        """{class: (ms, launches)} since create / reset (kernel_timing=True)."""
        t = N.cm_kernel_times()
        st = self._lib.cm_get_kernel_times(self._h, C.byref(t))
        N.raise_for(st, self._h)
        return {k: (t.ms[i], t.launches[i]) for i, k in enumerate(N.KERNEL_CLASSES)}

    def synchronize(self) -> None:
        N.raise_for(self._lib.cm_synchronize(self._h), self._h)
        self._inflight.clear()

    def reset(self) -> None:
        N.raise_for(self._lib.cm_reset(self._h), self._h)

    def device_bytes(self) -> int:
        return int(self._lib.cm_device_bytes(self._h))

    def stream_ptr(self) -> int:
        return int(self._lib.cm_stream(self._h) or 0)

    def close(self) -> None:
        if self._h:
            self._lib.cm_destroy(self._h)
            self._h = C.c_void_p()
        self._inflight = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Several engines whose frames run as one CUDA graph per staging round
    (cm_batch_*).  ``mode`` "fused" (default): when every system is in the
    ATOMS layout with the FP32 search, each stage of the chain is one kernel
    launch for all systems, draining a device work table of (system, block)
    entries; otherwise, or with "streams", each system's kernels run on its own
    stream, forked from and joined to one capture.  Counts are those of
    submitting to each engine alone.  Close the batch before its engines."""

    MODES = {"fused": 0, "streams": 1}

    def __init__(self, engines, mode: str = "fused"):
        self._lib = N.load()
        self.engines = list(engines)
        if mode not in self.MODES:
            raise ValueError(f"mode must be one of {sorted(self.MODES)}")
        arr = (C.c_void_p * len(self.engines))(*[e._h.value for e in self.engines])
        self._b = C.c_void_p()
        N.raise_for(self._lib.cm_batch_create(arr, len(self.engines), C.byref(self._b)), None)
        N.raise_for(self._lib.cm_batch_set_mode(self._b, self.MODES[mode]), None, batch=self._b)

    def submit(self, items) -> None:
        """``items[i]`` = (solute_xyz, solvent_xyz, cells[, frame_ids]) for
        engine i, or None to give it no frames in this call."""
        if len(items) != len(self.engines):
            raise ValueError("one item per engine")
        frs = (N.cm_frames * len(self.engines))()
        keeps = []
        for i, (e, it) in enumerate(zip(self.engines, items)):
            if it is None:
                continue
            xs, xv, cells = it[:3]
            ids = it[3] if len(it) > 3 else None
            fr, keep = frames_struct(xs, xv, cells, None, ids, e.Ns, e.Nv, e.autocorrelation)
            frs[i] = fr
            keeps.append(keep)
            e._inflight.append(keep)
        N.raise_for(self._lib.cm_batch_submit(self._b, frs), None, batch=self._b)

    def graph_stats(self) -> dict:
        a, b = C.c_int64(0), C.c_int64(0)
        N.raise_for(self._lib.cm_batch_graph_stats(self._b, C.byref(a), C.byref(b)), None, batch=self._b)
        r, l, n = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        N.raise_for(self._lib.cm_batch_fused_stats(self._b, C.byref(r), C.byref(l), C.byref(n)), None, batch=self._b)
        return {"graph_launches": a.value, "graph_instantiations": b.value, "fused_rounds": r.value,
                "stage_launches": l.value, "fused_systems": n.value}

    def close(self) -> None:
        if self._b:
            self._lib.cm_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


SNAPSHOT_COUNTS = ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
                   "solvent_group_random")


def save_snapshot(filename: str, snap: dict) -> str:
    """Write an engine snapshot (exact int64 half-unit counts and the frame
    weight, frames and volume sum behind them) as a compressed .npz."""
    np.savez_compressed(filename, **{k: np.asarray(snap[k]) for k in SNAPSHOT_COUNTS},
                        frame_weight=np.float64(snap["frame_weight"]), frames=np.int64(snap["frames"]),
                        volume_total=np.float64(snap["volume_total"]))
    return filename


def load_snapshot(filename: str) -> dict:
    """Read a snapshot written by ``save_snapshot``."""
    with np.load(filename, allow_pickle=False) as z:
        snap = {k: np.array(z[k], dtype=np.int64) for k in SNAPSHOT_COUNTS}
        snap.update(frame_weight=float(z["frame_weight"]), frames=int(z["frames"]), volume_total=float(z["volume_total"]))
    return snap
