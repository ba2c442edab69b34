"""ctypes wrapper of the CPU oracle (oracle/cm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the tests, by the smoke check and by
the CPU-baseline leg of the benchmark, always as the checker, never as the
thing measured for the GPU engine or shipped with it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


class orc_desc(C.Structure):
    _fields_ = [
        ("ms", C.c_int32), ("aps", C.c_int32), ("mv", C.c_int32), ("apv", C.c_int32),
        ("autocorrelation", C.c_int32), ("irefatom", C.c_int32),
        ("cutoff", C.c_double), ("binstep", C.c_double), ("dbulk", C.c_double),
        ("usecutoff", C.c_int32), ("nbins", C.c_int32), ("n_random_samples", C.c_int32),
        ("coordination_number_only", C.c_int32), ("seed", C.c_uint64),
        ("solute_ngroups", C.c_int32), ("solute_grp_off", C.POINTER(C.c_int64)), ("solute_grp", C.POINTER(C.c_int32)),
        ("solvent_ngroups", C.c_int32), ("solvent_grp_off", C.POINTER(C.c_int64)),
        ("solvent_grp", C.POINTER(C.c_int32)), ("backend", C.c_int32),
    ]


_LP = C.POINTER(C.c_int64)


class orc_counts(C.Structure):
    _fields_ = [("md", _LP), ("md_rand", _LP), ("rdf", _LP), ("rdf_rand", _LP), ("gs", _LP), ("gs_rand", _LP),
                ("gv", _LP), ("gv_rand", _LP), ("pairs_real", C.c_int64), ("pairs_rand", C.c_int64)]


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with the Makefile beside this file."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "cm_oracle.c")):
        r = subprocess.run(["make", "-C", HERE, "-B" if force else "all"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_frames.argtypes = [C.POINTER(orc_desc), C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                 C.POINTER(C.c_int64), C.c_int32, C.POINTER(orc_counts)]
        L.orc_frames.restype = C.c_int
        L.orc_setbin.argtypes = [C.c_double, C.c_double]
        L.orc_setbin.restype = C.c_int32
        L.orc_mindist2.argtypes = [C.POINTER(C.c_double)] * 3
        L.orc_mindist2.restype = C.c_double
        L.orc_cell_volume.argtypes = [C.POINTER(C.c_double)]
        L.orc_cell_volume.restype = C.c_double
        L.orc_eulermat_cs.argtypes = [C.c_double] * 6 + [C.POINTER(C.c_double)]
        L.orc_move.argtypes = [C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_stream_draws.argtypes = [C.c_uint64] * 5 + [C.c_int32, C.POINTER(C.c_uint64)]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def csr(rows, n):
    off = np.zeros(n + 1, dtype=np.int64)
    vals = []
    for i in range(n):
        off[i + 1] = off[i] + len(rows[i])
        vals.extend(rows[i])
    return off, np.asarray(vals if vals else [0], dtype=np.int32)


def default_groups(n, apm):
    return [[i % apm] for i in range(n)]


def run(*, ms, aps, mv, apv, autocorrelation, irefatom, cutoff, binstep, dbulk, usecutoff, nbins, n_random_samples,
        seed, solute_xyz, solvent_xyz, cells, frame_ids, coordination_number_only=False, solute_groups=None,
        solute_ngroups=0, solvent_groups=None, solvent_ngroups=0, backend="cells", nthreads=0):
    """Half-unit integer counts of all frames.  ``cells`` are [F, 3, 3]
    matrices whose columns are the lattice vectors; group tables as in the
    engine (None = per-atom-type groups)."""
    L = lib()
    d = orc_desc()
    d.ms, d.aps, d.mv, d.apv = ms, aps, mv, apv
    d.autocorrelation = int(bool(autocorrelation))
    d.irefatom = irefatom
    d.cutoff, d.binstep, d.dbulk = cutoff, binstep, dbulk
    d.usecutoff = int(bool(usecutoff))
    d.nbins = nbins
    d.n_random_samples = n_random_samples
    d.coordination_number_only = int(bool(coordination_number_only))
    d.seed = seed & 0xFFFFFFFFFFFFFFFF
    Nv = mv * apv
    if solute_groups is None:
        solute_groups, solute_ngroups = default_groups(aps, aps), aps
    if solvent_groups is None:
        solvent_groups, solvent_ngroups = default_groups(Nv, apv), apv
    so, si = csr(solute_groups, aps)
    vo, vi = csr(solvent_groups, Nv)
    d.solute_ngroups, d.solute_grp_off, d.solute_grp = solute_ngroups, so.ctypes.data_as(_LP), si.ctypes.data_as(C.POINTER(C.c_int32))
    d.solvent_ngroups, d.solvent_grp_off, d.solvent_grp = solvent_ngroups, vo.ctypes.data_as(_LP), vi.ctypes.data_as(C.POINTER(C.c_int32))
    d.backend = {"brute": 0, "cells": 1}[backend]
    xs = np.ascontiguousarray(solute_xyz, dtype=np.float64)
    nf = xs.shape[0]
    xv = None if solvent_xyz is None else np.ascontiguousarray(solvent_xyz, dtype=np.float64)
    cm = np.ascontiguousarray(np.transpose(np.asarray(cells, dtype=np.float64).reshape(nf, 3, 3), (0, 2, 1))).reshape(nf, 9)
    ids = np.ascontiguousarray(frame_ids, dtype=np.int64)
    gv = solvent_ngroups if not autocorrelation else max(solvent_ngroups, 1)
    out = {
        "md": np.zeros(nbins, np.int64), "md_random": np.zeros(nbins, np.int64),
        "rdf": np.zeros(nbins, np.int64), "rdf_random": np.zeros(nbins, np.int64),
        "solute_group": np.zeros((solute_ngroups, nbins), np.int64),
        "solute_group_random": np.zeros((solute_ngroups, nbins), np.int64),
        "solvent_group": np.zeros((gv, nbins), np.int64), "solvent_group_random": np.zeros((gv, nbins), np.int64),
    }
    c = orc_counts()
    for name, key in (("md", "md"), ("md_rand", "md_random"), ("rdf", "rdf"), ("rdf_rand", "rdf_random"),
                      ("gs", "solute_group"), ("gs_rand", "solute_group_random"), ("gv", "solvent_group"),
                      ("gv_rand", "solvent_group_random")):
        setattr(c, name, out[key].ctypes.data_as(_LP))
    st = L.orc_frames(C.byref(d), nf, xs.ctypes.data, None if xv is None else xv.ctypes.data, _dp(cm),
                      ids.ctypes.data_as(_LP), nthreads, C.byref(c))
    if st != 0:
        raise ValueError(f"oracle rejected the input (status {st})")
    if autocorrelation:
        out["solvent_group"][:] = 0
        out["solvent_group_random"][:] = 0
    out["pairs_real"] = c.pairs_real
    out["pairs_random"] = c.pairs_rand
    return out


def setbin(d, step):
    return lib().orc_setbin(d, step)


def mindist2(H, x, y):
    Hc = np.ascontiguousarray(np.asarray(H, dtype=np.float64).T).reshape(9)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return lib().orc_mindist2(_dp(Hc), _dp(x), _dp(y))


def cell_volume(H):
    """dot(cross(a, b), c) of a cell whose columns are a, b, c."""
    Hc = np.ascontiguousarray(np.asarray(H, dtype=np.float64).T).reshape(9)
    return lib().orc_cell_volume(_dp(Hc))


def stream_draws(seed, tag, a, b, c, n):
    out = np.zeros(n, dtype=np.uint64)
    lib().orc_stream_draws(seed, tag, a, b, c, n, out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return out


def eulermat_cs(c1, s1, c2, s2, c3, s3):
    A = np.zeros(9)
    lib().orc_eulermat_cs(c1, s1, c2, s2, c3, s3, _dp(A))
    return A.reshape(3, 3)


def move(x, newcm, A):
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    lib().orc_move(_dp(x), len(x), _dp(np.ascontiguousarray(newcm, dtype=np.float64)),
                   _dp(np.ascontiguousarray(A, dtype=np.float64).reshape(9)))
    return x


# ----------------------------------------------------------------- grid3D
def grid3d(solute_xyz, atom_type, table, d, *, dmin, dmax, step, chunk=2048, limit=None):
    """CPU restatement of grid3D's grid loop (src/tools/grid3D.jl:71-137),
    the checker of the engine's cm_grid3d.

    The grid spans the solute's bounding box (PDBTools.maxmin) widened by
    dmax, n = ceil((length + 2 dmax) / step + 1) points per axis, point
    (ix, iy, iz) at xmin - dmax + step (ix - 1), ...  Each point's closest
    solute atom (PDBTools.closest: Euclidean, no periodic images, the first
    atom at the minimum distance) is kept when dmin < r < dmax and the atom's
    contribution curve (``table[atom_type]`` over the bin distances ``d``),
    linearly interpolated at r, is positive.  Returns the kept points in loop
    order (ix outermost): linear index, 0-based solute atom, r and the value,
    plus n and the grid origin (``limit`` stops after that many points).
    """
    x = np.asarray(solute_xyz, dtype=np.float64)
    xmin = x.min(axis=0)
    xlen = x.max(axis=0) - xmin
    n = [int(math.ceil((xlen[k] + 2 * dmax) / step + 1)) for k in range(3)]
    origin = xmin - dmax
    table = np.asarray(table, dtype=np.float64)
    d = np.asarray(d, dtype=np.float64)
    atom_type = np.asarray(atom_type, dtype=np.int64)
    total = n[0] * n[1] * n[2] if limit is None else min(limit, n[0] * n[1] * n[2])
    pts, atoms, rs, vals = [], [], [], []
    for g0 in range(0, total, chunk):
        g = np.arange(g0, min(total, g0 + chunk), dtype=np.int64)
        ix, rem = np.divmod(g, n[1] * n[2])
        iy, iz = np.divmod(rem, n[2])
        p = np.stack([origin[k] + step * idx.astype(np.float64) for k, idx in enumerate((ix, iy, iz))], axis=1)
        dx = p[:, None, 0] - x[None, :, 0]
        dy = p[:, None, 1] - x[None, :, 1]
        dz = p[:, None, 2] - x[None, :, 2]
        d2 = (dx * dx + dy * dy) + dz * dz
        iat = np.argmin(d2, axis=1)              # first atom at the minimum
        r = np.sqrt(d2[np.arange(len(g)), iat])
        keep = (dmin < r) & (r < dmax)
        for j in np.nonzero(keep)[0]:
            c = table[atom_type[iat[j]]]
            iright = int(np.searchsorted(d, r[j], side="right"))   # first d > r
            ileft = iright - 1
            cr = c[ileft] + (c[iright] - c[ileft]) / (d[iright] - d[ileft]) * (r[j] - d[ileft])
            if cr > 0:
                pts.append(int(g[j]))
                atoms.append(int(iat[j]))
                rs.append(float(r[j]))
                vals.append(float(cr))
    return {"point": np.array(pts, dtype=np.int64), "atom": np.array(atoms, dtype=np.int32),
            "distance": np.array(rs), "value": np.array(vals), "n": n, "origin": origin, "evaluated": total}
