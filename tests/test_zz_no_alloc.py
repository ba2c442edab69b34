"""Allocation-free entry point cm_frame_counts_noalloc, called through the C ABI.

Its counts for one frame must equal, bit for bit, what cm_submit_frames +
cm_read_raw_counts give for a handle that was given only that frame, and the
oracle's.  Two calls in a row on different frames (and then on a different
system) check that each call clears the shared static scratch the previous
call left behind, and the device's free memory must not move while calls run
(the entry point exists for callers that cannot allocate).  The file is named
to be collected last, and passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

KEYS = ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
        "solvent_group_random")

OPT = dict(irefatom=1, cutoff=8.0, binstep=0.05, dbulk=8.0, usecutoff=False, nbins=200, n_random_samples=6, seed=17)


def system(rng, H, ms, aps, mv, apv, nframes, self_mode):
    def mols(n, apm):
        c = rng.random((n, 1, 3)) @ H.T
        return (c + rng.normal(scale=0.9, size=(n, apm, 3))).reshape(-1, 3)

    xs0 = mols(ms, aps)
    xv0 = None if self_mode else mols(mv, apv)
    xs = np.stack([xs0 + rng.normal(scale=0.2, size=xs0.shape) for _ in range(nframes)])
    xv = None if self_mode else np.stack([xv0 + rng.normal(scale=0.2, size=xv0.shape) for _ in range(nframes)])
    return xs, xv, np.repeat(H[None], nframes, axis=0)


def desc_of(N, *, ms, aps, mv, apv, self_mode, precision):
    d = N.cm_system_desc()
    d.api_version = N.CM_API_VERSION
    d.solute_nmols, d.solute_natomspermol = ms, aps
    d.solvent_nmols, d.solvent_natomspermol = mv, apv
    d.autocorrelation = 1 if self_mode else 0
    d.irefatom = OPT["irefatom"]
    d.cutoff, d.binstep, d.dbulk = OPT["cutoff"], OPT["binstep"], OPT["dbulk"]
    d.usecutoff = 0
    d.nbins = OPT["nbins"]
    d.n_random_samples = OPT["n_random_samples"]
    d.lcell = 1
    d.mode = N.CM_MODE_MDDF
    d.precision = N.CM_PRECISION_FP32_GUARD if precision == "fp32" else N.CM_PRECISION_FP64
    d.regime = N.CM_REGIME_PAIRS
    d.seed = OPT["seed"]
    return d


def counts_len(*, aps, apv, self_mode):
    nb = OPT["nbins"]
    return 4 * nb + 2 * aps * nb + (0 if self_mode else 2 * apv * nb)


def engine_counts(cm, *, ms, aps, mv, apv, self_mode, precision, xs, xv, cell, frame_id):
    eng = cm.Engine(solute_nmols=ms, solute_natomspermol=aps, solvent_nmols=mv, solvent_natomspermol=apv,
                    autocorrelation=self_mode, lcell=1, precision=precision, regime="pairs", **OPT)
    eng.submit(xs[None], None if xv is None else xv[None], cell[None], frame_ids=[frame_id])
    raw = eng.raw_counts()
    eng.close()
    parts = [raw[k].ravel() for k in KEYS[:6]]
    if not self_mode:
        parts += [raw[k].ravel() for k in KEYS[6:]]
    return np.concatenate(parts)


def device_inputs(xs, xv, n):
    """The call's device buffers (made by torch, outside the entry point)."""
    import torch

    xs_d = torch.from_numpy(np.ascontiguousarray(xs[None])).cuda()
    xv_d = None if xv is None else torch.from_numpy(np.ascontiguousarray(xv[None])).cuda()
    out = torch.full((n,), -7, dtype=torch.int64, device="cuda")  # overwritten by the call
    return xs_d, xv_d, out


def noalloc_counts(cm, *, ms, aps, mv, apv, self_mode, precision, xs, xv, cell, frame_id, bufs=None):
    import torch

    N = cm._native
    lib = N.load()
    d = desc_of(N, ms=ms, aps=aps, mv=mv, apv=apv, self_mode=self_mode, precision=precision)
    n = counts_len(aps=aps, apv=apv, self_mode=self_mode)
    xs_d, xv_d, out = bufs if bufs is not None else device_inputs(xs, xv, n)
    cm_cols = np.ascontiguousarray(cell.T).reshape(9)  # column-major: columns are lattice vectors
    ids = np.array([frame_id], dtype=np.int64)
    fr = N.cm_frames()
    fr.nframes = 1
    fr.coord_type = N.CM_COORD_F64
    fr.memory = N.CM_MEM_DEVICE
    fr.solute_xyz = C.c_void_p(xs_d.data_ptr())
    fr.solvent_xyz = C.c_void_p(xv_d.data_ptr()) if xv_d is not None else None
    fr.cells = N.as_ptr(cm_cols, C.c_double)
    fr.weights = None
    fr.frame_ids = N.as_ptr(ids, C.c_int64)
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.cm_frame_counts_noalloc(C.byref(d), C.byref(fr), C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_int64)),
                                     n, C.c_void_p(stream))
    N.raise_for(st, None)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_matches_engine_on_consecutive_calls(cm, gpu_ready):
    rng = np.random.default_rng(20261203)
    H = np.array([[30.0, 9.0, 0.0], [0.0, 27.0, 0.0], [0.0, 0.0, 29.0]])
    xs, _, cells = system(rng, H, 400, 3, 400, 3, 2, True)
    kw = dict(ms=400, aps=3, mv=400, apv=3, self_mode=True, precision="fp32", xv=None)
    got = []
    for k in range(2):  # two calls in a row: the second finds the first call's scratch contents
        a = noalloc_counts(cm, xs=xs[k], cell=cells[k], frame_id=k + 1, **kw)
        got.append(a)
    for k in range(2):
        b = engine_counts(cm, xs=xs[k], cell=cells[k], frame_id=k + 1, **kw)
        assert np.array_equal(got[k], b), k
        assert got[k][:OPT["nbins"]].sum() > 0
    assert not np.array_equal(got[0], got[1])


@pytest.mark.gpu
def test_noalloc_matches_oracle_bin_by_bin(cm, orc, gpu_ready):
    """A small cross system, both precisions: every bin equals the oracle's."""
    rng = np.random.default_rng(11)
    xs, xv, cells = system(rng, np.diag([24.0, 25.0, 26.0]), 20, 4, 200, 3, 1, False)
    ref = orc.run(ms=20, aps=4, mv=200, apv=3, solute_xyz=xs, solvent_xyz=xv, cells=cells, frame_ids=[5],
                  autocorrelation=False, **OPT)
    expect = np.concatenate([ref[k].ravel() for k in KEYS])
    assert expect[:OPT["nbins"]].sum() > 0
    for prec in ("fp32", "fp64"):
        got = noalloc_counts(cm, ms=20, aps=4, mv=200, apv=3, self_mode=False, precision=prec, xs=xs[0], xv=xv[0],
                             cell=cells[0], frame_id=5)
        assert np.array_equal(got, expect), prec


@pytest.mark.gpu
def test_noalloc_allocates_no_device_memory(cm, gpu_ready):
    """After a first call (which may load the library's kernels), further
    calls, one of them on a larger system, leave the device's free memory
    where it was: every input and output buffer is made before the reading."""
    import torch

    rng = np.random.default_rng(13)
    small = system(rng, np.diag([26.0, 28.0, 27.0]), 150, 3, 150, 3, 2, True)
    large = system(rng, np.diag([60.0, 62.0, 61.0]), 2000, 3, 2000, 3, 1, True)
    n = counts_len(aps=3, apv=3, self_mode=True)
    calls = [(150, small, 0), (150, small, 1), (2000, large, 0), (150, small, 0)]
    bufs = [device_inputs(sysd[0][k], None, n) for _, sysd, k in calls]
    out = []
    free0 = None
    for i, ((m, (xs, _, cells), k), b) in enumerate(zip(calls, bufs)):
        out.append(noalloc_counts(cm, ms=m, aps=3, mv=m, apv=3, self_mode=True, precision="fp32", xs=xs[k], xv=None,
                                  cell=cells[k], frame_id=k + 1, bufs=b))
        torch.cuda.synchronize()
        free = torch.cuda.mem_get_info()[0]
        if i == 0:
            free0 = free
        assert free == free0, (i, free0 - free)
    assert np.array_equal(out[0], out[3]) and out[2][:OPT["nbins"]].sum() > 0


@pytest.mark.gpu
def test_noalloc_cross_system_after_self(cm, gpu_ready):
    """A cross system after a self system (other buffer layout in the same
    scratch), in FP32 and FP64, orthorhombic and small (multi-image) boxes."""
    rng = np.random.default_rng(7)
    for H, prec in ((np.diag([26.0, 28.0, 27.0]), "fp32"), (np.diag([15.0, 16.0, 15.5]), "fp64"),
                    (np.diag([15.0, 16.0, 15.5]), "fp32")):
        xs, xv, cells = system(rng, H, 30, 5, 250, 3, 1, False)
        kw = dict(ms=30, aps=5, mv=250, apv=3, self_mode=False, precision=prec)
        a = noalloc_counts(cm, xs=xs[0], xv=xv[0], cell=cells[0], frame_id=3, **kw)
        b = engine_counts(cm, xs=xs[0], xv=xv[0], cell=cells[0], frame_id=3, **kw)
        assert np.array_equal(a, b), (prec, H[0, 0])


def test_noalloc_rejects_oversize_system(cm):
    """Systems whose buffers exceed the static scratch are refused before any
    CUDA call, with the size they would need."""
    N = cm._native
    lib = N.load()
    d = desc_of(N, ms=200000, aps=14, mv=200000, apv=14, self_mode=True, precision="fp32")
    fr = N.cm_frames()
    fr.nframes = 1
    fr.coord_type = N.CM_COORD_F32
    fr.memory = N.CM_MEM_DEVICE
    fr.solute_xyz = C.c_void_p(16)  # never dereferenced: the size check comes first
    cell = np.eye(3).reshape(9) * 300.0
    ids = np.array([1], dtype=np.int64)
    fr.cells = N.as_ptr(cell, C.c_double)
    fr.frame_ids = N.as_ptr(ids, C.c_int64)
    n = counts_len(aps=14, apv=14, self_mode=True)
    buf = np.zeros(n, dtype=np.int64)
    st = lib.cm_frame_counts_noalloc(C.byref(d), C.byref(fr), N.as_ptr(buf, C.c_int64), n, None)
    assert st == N.CM_EINVAL
    msg = lib.cm_last_error(None).decode()
    assert "bytes of scratch" in msg and str(N.CM_NOALLOC_SCRATCH_BYTES) in msg
