"""Frames given as slices of a larger array (cm_frames frame strides): each
frame's atoms contiguous, the frames further apart, read in place from device
memory and copied row by row from host memory.  The counts equal those of the
same frames given as one contiguous array, through the engine and through the
request server (which also takes device frames)."""
import numpy as np
import pytest

from helpers import KEYS, TRICLINIC, make_system

pytestmark = pytest.mark.gpu

SYS = dict(solute_nmols=50, solute_natomspermol=5, solvent_nmols=50, solvent_natomspermol=5, autocorrelation=True,
           irefatom=1, cutoff=7.0, binstep=0.02, dbulk=7.0, usecutoff=False, nbins=350, n_random_samples=4, seed=5)


def frames_in_a_larger_array(xs, extra=37):
    big = np.random.default_rng(9).random((xs.shape[0], xs.shape[1] + extra, 3)).astype(xs.dtype) * 500.0
    big[:, : xs.shape[1]] = xs
    return big


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_frame_slices_equal_contiguous_frames(cm, gpu_ready, precision):
    import torch

    rng = np.random.default_rng(61)
    xs, _, cells = make_system(rng, TRICLINIC, 50, 5, 50, 5, 5, True)
    xs = xs.astype(np.float32)
    big = frames_in_a_larger_array(xs)
    out = []
    for frames in (xs.copy(), big[:, :250], torch.from_numpy(big).cuda()[:, :250]):
        with cm.Engine(precision=precision, **SYS) as eng:
            eng.submit(frames, None, cells)
            out.append(eng.raw_counts())
    for k in KEYS[:6]:
        assert np.array_equal(out[0][k], out[1][k]), k
        assert np.array_equal(out[0][k], out[2][k]), k
    assert out[0]["md"].sum() > 0


def test_server_takes_device_frame_slices(cm, gpu_ready):
    import torch

    rng = np.random.default_rng(62)
    xs, _, cells = make_system(rng, TRICLINIC, 50, 5, 50, 5, 4, True)
    xs = xs.astype(np.float32)
    big = torch.from_numpy(frames_in_a_larger_array(xs)).cuda()
    with cm.Engine(precision="fp32", **SYS) as eng:
        eng.submit(xs, None, cells)
        want = eng.raw_counts()
    with cm.Server(frames_per_turn=2) as srv:
        rid = srv.submit(big[:, :250], None, cells, precision="fp32", **SYS)
        assert srv.wait(rid, timeout=120)["state"] == "done"
        got = srv.raw_counts(rid)
    for k in KEYS[:6]:
        assert np.array_equal(got[k], want[k]), k
