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


class Engine:
    """GPU engine handle.

    Parameters follow the reference's Options / AtomSelection / Result fields.
    ``solute_groups`` is a list, per atom of one solute molecule (local index),
    of the group numbers it credits; ``solvent_groups`` the same per atom of
    the whole solvent selection.  ``None`` means default per-atom-type groups.
    """

    def __init__(
        self,
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
    ):
        self._lib = N.load()
        self._h = C.c_void_p()
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
        self._keep = []
        if solute_groups is not None:
            off, idx = N.csr(solute_groups, solute_natomspermol)
            self._keep += [off, idx]
            d.solute_ngroups = solute_ngroups
            d.solute_group_offsets = N.as_ptr(off, C.c_int64)
            d.solute_groups = N.as_ptr(idx, C.c_int32)
        if solvent_groups is not None:
            off, idx = N.csr(solvent_groups, solvent_nmols * solvent_natomspermol)
            self._keep += [off, idx]
            d.solvent_ngroups = solvent_ngroups
            d.solvent_group_offsets = N.as_ptr(off, C.c_int64)
            d.solvent_groups = N.as_ptr(idx, C.c_int32)
        d.device = device
        d.max_frames_per_batch = max_frames_per_batch
        d.hbm_budget_bytes = hbm_budget_bytes
        d.kernel_timing = 1 if kernel_timing else 0
        st = self._lib.cm_create(C.byref(d), C.byref(self._h))
        N.raise_for(st, None)
        self.desc = d
        self.nbins = nbins
        self.ngroups_solute = solute_ngroups if solute_groups is not None else solute_natomspermol
        self.ngroups_solvent = solvent_ngroups if solvent_groups is not None else solvent_natomspermol
        self.autocorrelation = autocorrelation
        self.Ns = solute_nmols * solute_natomspermol
        self.Nv = solvent_nmols * solvent_natomspermol

    # -------------------------------------------------------------- frames
    def submit(self, solute_xyz, solvent_xyz, cells, weights=None, frame_ids=None) -> None:
        """Add frames.  Coordinates are [nframes, natoms, 3] float32/float64
        numpy arrays (host) or torch tensors (host or CUDA); cells are
        [nframes, 3, 3] matrices whose columns are the lattice vectors."""
        xs, kind_s, mem_s = self._coords(solute_xyz, self.Ns)
        nf = xs.shape[0] if not _is_torch(xs) else int(xs.shape[0])
        xv = None
        if not self.autocorrelation:
            xv, kind_v, mem_v = self._coords(solvent_xyz, self.Nv)
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
        fr.solute_xyz = self._ptr(xs)
        fr.solvent_xyz = self._ptr(xv) if xv is not None else None
        fr.cells = N.as_ptr(cm, C.c_double)
        fr.weights = N.as_ptr(w, C.c_double) if w is not None else None
        fr.frame_ids = N.as_ptr(ids, C.c_int64)
        st = self._lib.cm_submit_frames(self._h, C.byref(fr))
        N.raise_for(st, self._h)

    @staticmethod
    def _ptr(x):
        if x is None:
            return None
        if _is_torch(x):
            return C.c_void_p(x.data_ptr())
        return C.c_void_p(x.ctypes.data)

    @staticmethod
    def _coords(x, natoms):
        if _is_torch(x):
            import torch

            if x.dtype not in (torch.float32, torch.float64):
                raise ValueError("coordinates must be float32 or float64")
            x = x.contiguous()
            kind = N.CM_COORD_F32 if x.dtype == torch.float32 else N.CM_COORD_F64
            mem = N.CM_MEM_DEVICE if x.is_cuda else N.CM_MEM_HOST
            if x.dim() == 2:
                x = x.unsqueeze(0)
            if x.shape[1] != natoms or x.shape[2] != 3:
                raise ValueError(f"coordinates must be [nframes, {natoms}, 3]")
            return x, kind, mem
        a = np.asarray(x)
        if a.dtype not in (np.float32, np.float64):
            a = a.astype(np.float64)
        a = np.ascontiguousarray(a)
        if a.ndim == 2:
            a = a[None]
        if a.shape[1] != natoms or a.shape[2] != 3:
            raise ValueError(f"coordinates must be [nframes, {natoms}, 3]")
        return a, (N.CM_COORD_F32 if a.dtype == np.float32 else N.CM_COORD_F64), N.CM_MEM_HOST

    # -------------------------------------------------------------- output
    def counts(self) -> dict:
        """Frame-weighted counts (the Result fields before finalresults!)."""
        nb = self.nbins
        out = {
            "md_count": np.zeros(nb),
            "md_count_random": np.zeros(nb),
            "rdf_count": np.zeros(nb),
            "rdf_count_random": np.zeros(nb),
            "solute_group_count": np.zeros((self.ngroups_solute, nb)),
            "solute_group_count_random": np.zeros((self.ngroups_solute, nb)),
            "solvent_group_count": np.zeros((self.ngroups_solvent, nb)),
            "solvent_group_count_random": np.zeros((self.ngroups_solvent, nb)),
        }
        c = N.cm_counts()
        for k, v in out.items():
            setattr(c, k, N.as_ptr(v, C.c_double))
        st = self._lib.cm_read_counts(self._h, C.byref(c))
        N.raise_for(st, self._h)
        out["volume_total"] = c.volume_total
        out["weight_total"] = c.weight_total
        out["frames"] = c.frames
        return out

    def raw_counts(self) -> dict:
        """Exact int64 half-unit counts (runs with a single frame weight)."""
        nb = self.nbins
        out = {
            "md": np.zeros(nb, np.int64),
            "md_random": np.zeros(nb, np.int64),
            "rdf": np.zeros(nb, np.int64),
            "rdf_random": np.zeros(nb, np.int64),
            "solute_group": np.zeros((self.ngroups_solute, nb), np.int64),
            "solute_group_random": np.zeros((self.ngroups_solute, nb), np.int64),
            "solvent_group": np.zeros((self.ngroups_solvent, nb), np.int64),
            "solvent_group_random": np.zeros((self.ngroups_solvent, nb), np.int64),
        }
        c = N.cm_raw_counts()
        for k, v in out.items():
            setattr(c, k, N.as_ptr(v, C.c_int64))
        st = self._lib.cm_read_raw_counts(self._h, C.byref(c))
        N.raise_for(st, self._h)
        return out

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

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
