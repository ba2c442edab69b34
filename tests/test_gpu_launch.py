"""Captured-graph launch of compute chunks (launch="graph") against
one-launch-per-kernel stream launch: identical counts for both search
layouts, with chunks of changing shape (a short last chunk, growing cell
grids) that make the executable graph be updated in place or rebuilt, and
against the CPU oracle."""
import numpy as np
import pytest


pytestmark = pytest.mark.gpu

KEYS = ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
        "solvent_group_random")
OPT = dict(irefatom=1, cutoff=7.0, binstep=0.05, dbulk=7.0, usecutoff=False, nbins=140, n_random_samples=3, seed=5)


def system(rng, ms, aps, mv, apv, nframes, self_mode, grow=False):
    H0 = np.array([[26.0, 8.0, 0.0], [0.0, 24.0, 0.0], [0.0, 0.0, 25.0]])
    cells = np.stack([H0 * (1.0 + (0.02 * k if grow else 0.0)) for k in range(nframes)])

    def mols(n, apm):
        c = rng.random((n, 1, 3)) @ H0.T
        return (c + rng.normal(scale=0.9, size=(n, apm, 3))).reshape(-1, 3)

    xs0 = mols(ms, aps)
    xv0 = None if self_mode else mols(mv, apv)
    xs = np.stack([xs0 + rng.normal(scale=0.2, size=xs0.shape) for _ in range(nframes)])
    xv = None if self_mode else np.stack([xv0 + rng.normal(scale=0.2, size=xv0.shape) for _ in range(nframes)])
    return xs, xv, cells


def run(cm, launch, xs, xv, cells, **kw):
    eng = cm.Engine(launch=launch, **kw)
    eng.submit(xs, xv, cells)
    out = eng.raw_counts()
    st = eng.stats()
    eng.close()
    return out, st


@pytest.mark.parametrize("case", ["pairs-self", "pairs-cross", "atoms-cross"])
@pytest.mark.parametrize("grow", [False, True], ids=["fixed-cell", "growing-cell"])
def test_graph_launch_matches_stream_launch(cm, orc, case, grow):
    rng = np.random.default_rng({"pairs-self": 11, "pairs-cross": 12, "atoms-cross": 13}[case] * 2 + int(grow))
    if case == "pairs-self":
        ms, aps, mv, apv, self_mode, regime = 400, 5, 400, 5, True, "pairs"
    elif case == "pairs-cross":
        ms, aps, mv, apv, self_mode, regime = 30, 6, 700, 3, False, "pairs"
    else:
        ms, aps, mv, apv, self_mode, regime = 1, 80, 700, 3, False, "atoms"
    nframes = 11  # chunks of 4, 4 and 3 frames: the last one changes the chain's shape
    xs, xv, cells = system(rng, ms, aps, mv, apv, nframes, self_mode, grow)
    kw = dict(solute_nmols=ms, solute_natomspermol=aps, solvent_nmols=mv, solvent_natomspermol=apv,
              autocorrelation=self_mode, precision="fp32", regime=regime, max_frames_per_batch=4, **OPT)
    g, gst = run(cm, "graph", xs, xv, cells, **kw)
    s, sst = run(cm, "stream", xs, xv, cells, **kw)
    for k in KEYS:
        assert np.array_equal(g[k], s[k]), k
    assert gst["graph_launches"] >= 3 and sst["graph_launches"] == 0
    assert 1 <= gst["graph_instantiations"] < gst["graph_launches"]
    ref = orc.run(ms=ms, aps=aps, mv=mv, apv=apv, solute_xyz=xs, solvent_xyz=xv, cells=cells,
                  frame_ids=list(range(1, nframes + 1)), backend="cells", autocorrelation=self_mode, **OPT)
    for k in KEYS:
        if self_mode and k.startswith("solvent"):
            continue
        assert np.array_equal(np.asarray(g[k]).ravel(), np.asarray(ref[k]).ravel()), k



def test_batch_graph_counts_equal_each_system_alone(cm):
    """Systems of both layouts, precisions and uneven frame counts (one that
    needs two staging rounds, one that sits a call out) submitted as a batch
    in two calls give, per system, the counts of an engine of its own."""
    rng = np.random.default_rng(31)
    specs = [  # (ms, aps, mv, apv, self, regime, precision, nframes first call, second call)
        (300, 4, 300, 4, True, "pairs", "fp32", 5, 3),
        (20, 6, 500, 3, False, "pairs", "fp32", 9, 0),
        (1, 70, 600, 3, False, "atoms", "fp32", 4, 4),
        (200, 3, 200, 3, True, "pairs", "fp64", 2, 6),
    ]
    systems, engines, alone = [], [], []
    for ms, aps, mv, apv, self_mode, regime, prec, n1, n2 in specs:
        xs, xv, cells = system(rng, ms, aps, mv, apv, n1 + n2, self_mode)
        kw = dict(solute_nmols=ms, solute_natomspermol=aps, solvent_nmols=mv, solvent_natomspermol=apv,
                  autocorrelation=self_mode, precision=prec, regime=regime, max_frames_per_batch=4, **OPT)
        systems.append((xs, xv, cells, n1, n2))
        engines.append(cm.Engine(**kw))
        alone.append(run(cm, "stream", xs, xv, cells, **kw)[0])

    def part(k, lo, hi):
        xs, xv, cells = systems[k][:3]
        if hi == lo:
            return None
        return (xs[lo:hi], None if xv is None else xv[lo:hi], cells[lo:hi], np.arange(lo + 1, hi + 1))

    with cm.Batch(engines) as b:
        b.submit([part(k, 0, s[3]) for k, s in enumerate(systems)])
        b.submit([part(k, s[3], s[3] + s[4]) for k, s in enumerate(systems)])
        st = b.graph_stats()
    assert st["graph_launches"] >= 3 and st["graph_instantiations"] <= st["graph_launches"]
    for k, e in enumerate(engines):
        got = e.raw_counts()
        e.close()
        for key in KEYS:
            assert np.array_equal(got[key], alone[k][key]), (k, key)


@pytest.mark.parametrize("batched", [False, True], ids=["engine", "batch"])
def test_device_frames_then_host_frames(cm, batched):
    """A handle whose first frames come from device memory stages later
    host-memory frames too (its staging buffers are made on first use), alone
    and inside a batch; the counts equal one host-memory submit of all frames."""
    import torch

    rng = np.random.default_rng(47)
    xs, xv, cells = system(rng, 25, 6, 500, 3, 8, False)
    xs, xv = xs.astype(np.float32), xv.astype(np.float32)
    kw = dict(solute_nmols=25, solute_natomspermol=6, solvent_nmols=500, solvent_natomspermol=3, autocorrelation=False,
              precision="fp32", regime="pairs", max_frames_per_batch=4, **OPT)
    want = run(cm, "stream", xs, xv, cells, **kw)[0]
    ids = np.arange(1, 9)
    first = (torch.from_numpy(xs[:4]).cuda(), torch.from_numpy(xv[:4]).cuda(), cells[:4], ids[:4])
    second = (xs[4:], xv[4:], cells[4:], ids[4:])
    eng = cm.Engine(**kw)
    if batched:
        with cm.Batch([eng]) as b:
            b.submit([first])
            b.submit([second])
    else:
        eng.submit(*first[:3], frame_ids=first[3])
        eng.submit(*second[:3], frame_ids=second[3])
    got = eng.raw_counts()
    eng.close()
    for k in KEYS:
        assert np.array_equal(got[k], want[k]), k
