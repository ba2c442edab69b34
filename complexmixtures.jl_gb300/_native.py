"""ctypes binding of libcmgpu.so, the C ABI declared in include/cmgpu.h.

The shared library is the only compute path of this package: if it cannot be
loaded (not built, or no CUDA driver), every entry point that needs it raises
``NativeUnavailable``.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

CM_API_VERSION = 4
CM_OK, CM_EINVAL, CM_ENOMEM, CM_ECUDA, CM_EDEVICE, CM_ESTATE = range(6)
CM_MODE_MDDF, CM_MODE_COORDINATION_NUMBER = 0, 1
CM_PRECISION_FP64, CM_PRECISION_FP32_GUARD = 0, 1
CM_REGIME_AUTO, CM_REGIME_PAIRS, CM_REGIME_ATOMS = 0, 1, 2
CM_LAUNCH_AUTO, CM_LAUNCH_STREAM, CM_LAUNCH_GRAPH = 0, 1, 2
CM_SCHED_AUTO, CM_SCHED_CELL, CM_SCHED_BALANCED = 0, 1, 2
CM_REAL_AUTO, CM_REAL_WARP, CM_REAL_TILE = 0, 1, 2
CM_COORD_F64, CM_COORD_F32, CM_COORD_DCD = 0, 1, 2
CM_MEM_HOST, CM_MEM_DEVICE = 0, 1
CM_NOALLOC_SCRATCH_BYTES = 32 << 20
CM_NOALLOC_MAX_SAMPLES = 4096

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libcmgpu.so")


class NativeUnavailable(RuntimeError):
    """The CUDA engine library is missing or cannot be loaded."""


class cm_system_desc(C.Structure):
    _fields_ = [
        ("api_version", C.c_int32),
        ("solute_nmols", C.c_int32),
        ("solute_natomspermol", C.c_int32),
        ("solvent_nmols", C.c_int32),
        ("solvent_natomspermol", C.c_int32),
        ("autocorrelation", C.c_int32),
        ("irefatom", C.c_int32),
        ("cutoff", C.c_double),
        ("binstep", C.c_double),
        ("dbulk", C.c_double),
        ("usecutoff", C.c_int32),
        ("nbins", C.c_int32),
        ("n_random_samples", C.c_int32),
        ("lcell", C.c_int32),
        ("mode", C.c_int32),
        ("precision", C.c_int32),
        ("regime", C.c_int32),
        ("seed", C.c_uint64),
        ("solute_ngroups", C.c_int32),
        ("solute_group_offsets", C.POINTER(C.c_int64)),
        ("solute_groups", C.POINTER(C.c_int32)),
        ("solvent_ngroups", C.c_int32),
        ("solvent_group_offsets", C.POINTER(C.c_int64)),
        ("solvent_groups", C.POINTER(C.c_int32)),
        ("device", C.c_int32),
        ("max_frames_per_batch", C.c_int32),
        ("hbm_budget_bytes", C.c_int64),
        ("kernel_timing", C.c_int32),
        ("cell_scale_pct", C.c_int32),
        ("launch", C.c_int32),
        ("atoms_schedule", C.c_int32),
        ("guard_queue_capacity", C.c_int32),
        ("real_pass", C.c_int32),
        ("atoms_grid", C.c_int32),
        ("atoms_grid_capacity", C.c_int32),
    ]


class cm_dcd_layout(C.Structure):
    _fields_ = [
        ("natoms", C.c_int64),
        ("frame_bytes", C.c_int64),
        ("x_offset", C.c_int64),
        ("y_offset", C.c_int64),
        ("z_offset", C.c_int64),
        ("big_endian", C.c_int32),
        ("reserved", C.c_int32),
        ("solute_atoms", C.POINTER(C.c_int32)),
        ("solvent_atoms", C.POINTER(C.c_int32)),
    ]


class cm_frames(C.Structure):
    _fields_ = [
        ("nframes", C.c_int32),
        ("coord_type", C.c_int32),
        ("memory", C.c_int32),
        ("reserved", C.c_int32),
        ("solute_xyz", C.c_void_p),
        ("solvent_xyz", C.c_void_p),
        ("cells", C.POINTER(C.c_double)),
        ("weights", C.POINTER(C.c_double)),
        ("frame_ids", C.POINTER(C.c_int64)),
        ("solute_frame_stride", C.c_int64),
        ("solvent_frame_stride", C.c_int64),
    ]


_DP = C.POINTER(C.c_double)
_LP = C.POINTER(C.c_int64)


class cm_counts(C.Structure):
    _fields_ = [
        ("md_count", _DP),
        ("md_count_random", _DP),
        ("rdf_count", _DP),
        ("rdf_count_random", _DP),
        ("solute_group_count", _DP),
        ("solute_group_count_random", _DP),
        ("solvent_group_count", _DP),
        ("solvent_group_count_random", _DP),
        ("volume_total", C.c_double),
        ("weight_total", C.c_double),
        ("frames", C.c_int64),
    ]


class cm_raw_counts(C.Structure):
    _fields_ = [
        ("md", _LP),
        ("md_random", _LP),
        ("rdf", _LP),
        ("rdf_random", _LP),
        ("solute_group", _LP),
        ("solute_group_random", _LP),
        ("solvent_group", _LP),
        ("solvent_group_random", _LP),
    ]


RESULT_VECTORS = ("d", "md_count", "md_count_random", "coordination_number", "coordination_number_random", "mddf", "kb",
                  "rdf_count", "rdf_count_random", "sum_rdf_count", "sum_rdf_count_random", "rdf", "kb_rdf",
                  "volume_shell")
RESULT_GROUPS = ("solute_group_count", "solute_group_count_random", "solvent_group_count", "solvent_group_count_random")
RESULT_SCALARS = ("volume_total", "volume_bulk", "volume_domain", "density_solute", "density_solvent",
                  "density_solvent_bulk", "density_fix")


class cm_results(C.Structure):
    _fields_ = ([(k, C.POINTER(C.c_double)) for k in RESULT_VECTORS + RESULT_GROUPS]
                + [(k, C.c_double) for k in RESULT_SCALARS] + [("zero_random_bins", C.c_int64)])


class cm_contrib_query(C.Structure):
    _fields_ = [("side", C.c_int32), ("type", C.c_int32), ("divide", C.c_int32), ("nterms", C.c_int32),
                ("groups", C.POINTER(C.c_int32))]


CM_GROUP_SOLUTE, CM_GROUP_SOLVENT = 0, 1
CM_CONTRIB_TYPES = {"mddf": 0, "coordination_number": 1, "md_count": 2, "kbi": 3}


class cm_grid3d_desc(C.Structure):
    _fields_ = [
        ("device", C.c_int32), ("nbins", C.c_int32), ("natoms", C.c_int64), ("xyz", C.POINTER(C.c_double)),
        ("atom_type", C.POINTER(C.c_int32)), ("ntypes", C.c_int32), ("reserved", C.c_int32),
        ("table", C.POINTER(C.c_double)), ("d", C.POINTER(C.c_double)), ("dmin", C.c_double), ("dmax", C.c_double),
        ("step", C.c_double),
    ]


class cm_grid3d_out(C.Structure):
    _fields_ = [
        ("capacity", C.c_int64), ("count", C.c_int64), ("n", C.c_int64 * 3), ("origin", C.c_double * 3),
        ("point", C.POINTER(C.c_int64)), ("atom", C.POINTER(C.c_int32)), ("distance", C.POINTER(C.c_double)),
        ("value", C.POINTER(C.c_double)),
    ]


class cm_stats(C.Structure):
    _fields_ = [
        ("frames", C.c_int64),
        ("molecule_pairs_evaluated", C.c_int64),
        ("atom_pairs_evaluated", C.c_int64),
        ("hits_real", C.c_int64),
        ("hits_random", C.c_int64),
        ("guard_reevaluations", C.c_int64),
        ("guard_pair_evaluations", C.c_int64),
        ("max_guard_error", C.c_double),
        ("guard_band", C.c_double),
        ("regime", C.c_int32),
        ("kernels_per_frame", C.c_int32),
        ("kernel_launches", C.c_int64),
        ("graph_launches", C.c_int64),
        ("graph_instantiations", C.c_int64),
    ]


KERNEL_CLASSES = ("prep", "cells", "real", "bulk", "random", "other", "guard")


class cm_kernel_times(C.Structure):
    _fields_ = [("ms", C.c_double * 7), ("launches", C.c_int64 * 7)]


CM_TUNE_MAX = 8


class cm_tuning(C.Structure):
    _fields_ = [
        ("cell_scale_pct", C.c_int32),
        ("ncandidates", C.c_int32),
        ("candidates", C.c_int32 * CM_TUNE_MAX),
        ("ms_per_frame", C.c_double * CM_TUNE_MAX),
        ("atoms_schedule", C.c_int32),
        ("schedules", C.c_int32 * CM_TUNE_MAX),
        ("real_pass", C.c_int32),
        ("atoms_grid", C.c_int32),
        ("grids", C.c_int32 * CM_TUNE_MAX),
    ]


class cm_server_desc(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("max_active", C.c_int32),
        ("hbm_budget_bytes", C.c_int64),
        ("frames_per_turn", C.c_int32),
        ("reserved", C.c_int32),
    ]


class cm_request_info(C.Structure):
    _fields_ = [
        ("state", C.c_int32),
        ("status", C.c_int32),
        ("t_submit", C.c_double),
        ("t_admit", C.c_double),
        ("t_done", C.c_double),
        ("frames_submitted", C.c_int64),
        ("device_bytes", C.c_int64),
    ]


CM_REQ_QUEUED, CM_REQ_RUNNING, CM_REQ_DONE, CM_REQ_FAILED, CM_REQ_CANCELLED = range(5)

EXPORTED = (
    "cm_create",
    "cm_submit_frames",
    "cm_synchronize",
    "cm_set_dcd_layout",
    "cm_batch_create",
    "cm_batch_submit",
    "cm_batch_graph_stats",
    "cm_batch_set_mode",
    "cm_batch_fused_stats",
    "cm_batch_destroy",
    "cm_batch_last_error",
    "cm_read_counts",
    "cm_read_raw_counts",
    "cm_raw_counts_weight",
    "cm_load_raw_counts",
    "cm_read_results",
    "cm_contributions",
    "cm_get_stats",
    "cm_get_kernel_times",
    "cm_reset",
    "cm_destroy",
    "cm_last_error",
    "cm_status_string",
    "cm_device_bytes",
    "cm_memory_cache",
    "cm_grid3d",
    "cm_stream",
    "cm_measure_fp32_peak",
    "cm_frame_counts_noalloc",
    "cm_autotune",
    "cm_server_create",
    "cm_server_submit",
    "cm_server_poll",
    "cm_server_wait",
    "cm_server_read_counts",
    "cm_server_read_raw_counts",
    "cm_server_cancel",
    "cm_server_release",
    "cm_server_destroy",
    "cm_server_last_error",
)

_lib: Optional[C.CDLL] = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libcmgpu.so and declare the prototypes of include/cmgpu.h."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise NativeUnavailable(
            f"{path} not found: build the CUDA engine first (python -c 'import __graft_entry__ as g; g.build()')"
        )
    try:
        lib = C.CDLL(path)
    except OSError as e:  # missing libcudart / driver
        raise NativeUnavailable(f"cannot load {path}: {e}") from e
    H = C.c_void_p
    lib.cm_create.argtypes = [C.POINTER(cm_system_desc), C.POINTER(H)]
    lib.cm_create.restype = C.c_int
    lib.cm_submit_frames.argtypes = [H, C.POINTER(cm_frames)]
    lib.cm_submit_frames.restype = C.c_int
    lib.cm_synchronize.argtypes = [H]
    lib.cm_synchronize.restype = C.c_int
    lib.cm_read_counts.argtypes = [H, C.POINTER(cm_counts)]
    lib.cm_read_counts.restype = C.c_int
    lib.cm_read_raw_counts.argtypes = [H, C.POINTER(cm_raw_counts)]
    lib.cm_read_raw_counts.restype = C.c_int
    lib.cm_raw_counts_weight.argtypes = [H, C.POINTER(C.c_double)]
    lib.cm_raw_counts_weight.restype = C.c_int
    lib.cm_load_raw_counts.argtypes = [H, C.POINTER(cm_raw_counts), C.c_double, C.c_int64, C.c_double]
    lib.cm_load_raw_counts.restype = C.c_int
    lib.cm_get_stats.argtypes = [H, C.POINTER(cm_stats)]
    lib.cm_get_stats.restype = C.c_int
    lib.cm_get_kernel_times.argtypes = [H, C.POINTER(cm_kernel_times)]
    lib.cm_get_kernel_times.restype = C.c_int
    lib.cm_reset.argtypes = [H]
    lib.cm_reset.restype = C.c_int
    lib.cm_destroy.argtypes = [H]
    lib.cm_destroy.restype = C.c_int
    lib.cm_last_error.argtypes = [H]
    lib.cm_last_error.restype = C.c_char_p
    lib.cm_status_string.argtypes = [C.c_int]
    lib.cm_status_string.restype = C.c_char_p
    lib.cm_device_bytes.argtypes = [H]
    lib.cm_device_bytes.restype = C.c_int64
    lib.cm_read_results.argtypes = [H, C.c_double, C.POINTER(cm_results)]
    lib.cm_read_results.restype = C.c_int
    lib.cm_contributions.argtypes = [H, C.c_double, C.c_int32, C.POINTER(cm_contrib_query), C.POINTER(C.c_double)]
    lib.cm_contributions.restype = C.c_int
    lib.cm_set_dcd_layout.argtypes = [H, C.POINTER(cm_dcd_layout)]
    lib.cm_set_dcd_layout.restype = C.c_int
    lib.cm_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]
    lib.cm_batch_create.restype = C.c_int
    lib.cm_batch_submit.argtypes = [C.c_void_p, C.POINTER(cm_frames)]
    lib.cm_batch_submit.restype = C.c_int
    lib.cm_batch_graph_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.cm_batch_graph_stats.restype = C.c_int
    lib.cm_batch_set_mode.argtypes = [C.c_void_p, C.c_int32]
    lib.cm_batch_set_mode.restype = C.c_int
    lib.cm_batch_fused_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.cm_batch_fused_stats.restype = C.c_int
    lib.cm_batch_destroy.argtypes = [C.c_void_p]
    lib.cm_batch_destroy.restype = C.c_int
    lib.cm_batch_last_error.argtypes = [C.c_void_p]
    lib.cm_batch_last_error.restype = C.c_char_p
    lib.cm_grid3d.argtypes = [C.POINTER(cm_grid3d_desc), C.POINTER(cm_grid3d_out)]
    lib.cm_grid3d.restype = C.c_int
    lib.cm_memory_cache.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.cm_memory_cache.restype = C.c_int
    lib.cm_stream.argtypes = [H]
    lib.cm_stream.restype = C.c_void_p
    lib.cm_measure_fp32_peak.argtypes = [C.c_int32, C.c_double, C.POINTER(C.c_double)]
    lib.cm_measure_fp32_peak.restype = C.c_int
    lib.cm_frame_counts_noalloc.argtypes = [C.POINTER(cm_system_desc), C.POINTER(cm_frames), C.POINTER(C.c_int64),
                                            C.c_int64, C.c_void_p]
    lib.cm_frame_counts_noalloc.restype = C.c_int
    lib.cm_autotune.argtypes = [C.POINTER(cm_system_desc), C.POINTER(cm_frames), C.POINTER(cm_tuning)]
    lib.cm_autotune.restype = C.c_int
    S = C.c_void_p
    lib.cm_server_create.argtypes = [C.POINTER(cm_server_desc), C.POINTER(S)]
    lib.cm_server_submit.argtypes = [S, C.POINTER(cm_system_desc), C.POINTER(cm_frames), C.POINTER(C.c_int64)]
    lib.cm_server_poll.argtypes = [S, C.c_int64, C.POINTER(cm_request_info)]
    lib.cm_server_wait.argtypes = [S, C.c_int64, C.c_double, C.POINTER(cm_request_info)]
    lib.cm_server_read_counts.argtypes = [S, C.c_int64, C.POINTER(cm_counts)]
    lib.cm_server_read_raw_counts.argtypes = [S, C.c_int64, C.POINTER(cm_raw_counts)]
    lib.cm_server_cancel.argtypes = [S, C.c_int64]
    lib.cm_server_release.argtypes = [S, C.c_int64]
    lib.cm_server_destroy.argtypes = [S]
    for f in ("cm_server_create", "cm_server_submit", "cm_server_poll", "cm_server_wait", "cm_server_read_counts",
              "cm_server_read_raw_counts", "cm_server_cancel", "cm_server_release", "cm_server_destroy"):
        getattr(lib, f).restype = C.c_int
    lib.cm_server_last_error.argtypes = [S]
    lib.cm_server_last_error.restype = C.c_char_p
    _lib = lib
    return lib


def raise_for(status: int, handle, server=None, batch=None) -> None:
    """Turn a cm_status into the exception the reference raises for it."""
    if status == CM_OK:
        return
    lib = load()
    if server is not None:
        msg = lib.cm_server_last_error(server).decode(errors="replace")
    elif batch is not None:
        msg = lib.cm_batch_last_error(batch).decode(errors="replace")
    else:
        msg = lib.cm_last_error(handle).decode(errors="replace")
    what = lib.cm_status_string(status).decode()
    text = f"{what}: {msg}" if msg else what
    if status == CM_EINVAL:
        raise ValueError(text)
    if status == CM_ENOMEM:
        raise MemoryError(text)
    raise RuntimeError(text)


def csr(rows, nrows: int):
    """(offsets int64[nrows+1], values int32[]) from a list of int sequences."""
    off = np.zeros(nrows + 1, dtype=np.int64)
    vals = []
    for i in range(nrows):
        r = rows[i]
        off[i + 1] = off[i] + len(r)
        vals.extend(int(g) for g in r)
    return off, np.asarray(vals if vals else [0], dtype=np.int32)


def as_ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def measure_fp32_peak(device: int = 0, ms_target: float = 200.0) -> float:
    """FP32 CUDA-core TFLOP/s of a device (see cm_measure_fp32_peak)."""
    lib = load()
    out = C.c_double(0.0)
    raise_for(lib.cm_measure_fp32_peak(device, ms_target, C.byref(out)), None)
    return out.value
