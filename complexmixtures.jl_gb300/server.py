"""Request server: continuous batching of MDDF jobs on one GPU.

Wraps the cm_server_* entry points of libcmgpu.so.  Each request is one system
(the keyword arguments of ``Engine``) with its frames in host memory; the
server admits requests by device-memory budget, runs the admitted ones
concurrently on the device, and keeps each request's counts until released.
A request's counts equal those of an ``Engine`` given the same system and
frames alone.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _native as N
from .engine import counts_arrays, frames_struct, raw_arrays, system_desc

STATES = {N.CM_REQ_QUEUED: "queued", N.CM_REQ_RUNNING: "running", N.CM_REQ_DONE: "done", N.CM_REQ_FAILED: "failed",
          N.CM_REQ_CANCELLED: "cancelled"}


class Server:
    """A request server on one device.

    ``max_active``: requests on the device at once (0: no limit);
    ``hbm_budget_bytes``: device memory for admitted requests (0: no budget);
    ``frames_per_turn``: frames a request submits per scheduling turn.
    """

    def __init__(self, device: int = 0, max_active: int = 0, hbm_budget_bytes: int = 0, frames_per_turn: int = 32):
        self._lib = N.load()
        d = N.cm_server_desc()
        d.device = device
        d.max_active = max_active
        d.hbm_budget_bytes = hbm_budget_bytes
        d.frames_per_turn = frames_per_turn
        self._s = C.c_void_p()
        N.raise_for(self._lib.cm_server_create(C.byref(d), C.byref(self._s)), None, server=C.c_void_p())
        self._req = {}   # id -> (arrays kept alive, nbins, ngroups solute, ngroups solvent)

    def submit(self, solute_xyz, solvent_xyz, cells, weights=None, frame_ids=None, **system) -> int:
        """Queue a request; returns its id.  Coordinates are [nframes, natoms,
        3] float32 or float64 arrays: numpy, or torch tensors on the host or
        the GPU (kept alive, and not to be changed, until the request is
        done).  A frame may be a slice of a larger array (frames[:, :n]): the
        frame stride is passed, the frames are not copied."""
        d, keep_d = system_desc(**system)
        Ns = d.solute_nmols * d.solute_natomspermol
        Nv = d.solvent_nmols * d.solvent_natomspermol
        fr, keep_f = frames_struct(solute_xyz, solvent_xyz, cells, weights, frame_ids, Ns, Nv, bool(d.autocorrelation))
        rid = C.c_int64()
        self._check(self._lib.cm_server_submit(self._s, C.byref(d), C.byref(fr), C.byref(rid)))
        gs = d.solute_ngroups if system.get("solute_groups") is not None else d.solute_natomspermol
        gv = d.solvent_ngroups if system.get("solvent_groups") is not None else d.solvent_natomspermol
        self._req[rid.value] = (keep_d + keep_f, d.nbins, gs, gv)
        return rid.value

    def _check(self, st):
        N.raise_for(st, None, server=self._s)

    @staticmethod
    def _info(i: N.cm_request_info) -> dict:
        return {"state": STATES[i.state], "status": i.status, "t_submit": i.t_submit, "t_admit": i.t_admit,
                "t_done": i.t_done, "frames_submitted": i.frames_submitted, "device_bytes": i.device_bytes}

    def poll(self, rid: int) -> dict:
        i = N.cm_request_info()
        self._check(self._lib.cm_server_poll(self._s, rid, C.byref(i)))
        return self._info(i)

    def wait(self, rid: int, timeout: Optional[float] = None) -> dict:
        i = N.cm_request_info()
        self._check(self._lib.cm_server_wait(self._s, rid, -1.0 if timeout is None else float(timeout), C.byref(i)))
        return self._info(i)

    def counts(self, rid: int) -> dict:
        _, nb, gs, gv = self._req[rid]
        out, c = counts_arrays(nb, gs, gv)
        self._check(self._lib.cm_server_read_counts(self._s, rid, C.byref(c)))
        out["volume_total"] = c.volume_total
        out["weight_total"] = c.weight_total
        out["frames"] = c.frames
        return out

    def raw_counts(self, rid: int) -> dict:
        _, nb, gs, gv = self._req[rid]
        out, c = raw_arrays(nb, gs, gv)
        self._check(self._lib.cm_server_read_raw_counts(self._s, rid, C.byref(c)))
        return out

    def cancel(self, rid: int) -> None:
        self._check(self._lib.cm_server_cancel(self._s, rid))

    def release(self, rid: int) -> None:
        self._check(self._lib.cm_server_release(self._s, rid))
        self._req.pop(rid, None)

    def close(self) -> None:
        if self._s:
            self._lib.cm_server_destroy(self._s)
            self._s = C.c_void_p()
        self._req.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def latency_percentiles(infos, qs=(50, 99)) -> dict:
    """Percentiles (ms) of submit-to-done latency over request infos."""
    lat = np.array([1e3 * (i["t_done"] - i["t_submit"]) for i in infos if i["state"] == "done"])
    if lat.size == 0:
        return {f"p{q}": None for q in qs}
    return {f"p{q}": float(np.percentile(lat, q)) for q in qs}
