"""Fused batches (cm_batch in FUSED mode): every stage of a round is one
kernel launch for all systems, draining a device work table of (system,
block) entries.  Per system the counts must equal an engine of its own and
the CPU oracle; systems of uneven size, frame counts and chunk counts, with
the candidate grid and with the stencil walk, and a round that cannot be
fused (mixed layouts) falling back to per-system streams."""
import numpy as np
import pytest

from helpers import KEYS

pytestmark = pytest.mark.gpu

OPT = dict(irefatom=1, cutoff=6.0, binstep=0.05, dbulk=6.0, usecutoff=False, nbins=120, n_random_samples=4, seed=7)


def chain_system(rng, n_solute, n_water, nframes, box):
    H = np.diag([box, box, box])
    steps = rng.normal(size=(n_solute, 3))
    chain = np.cumsum(steps / np.linalg.norm(steps, axis=1, keepdims=True) * 1.53, axis=0)
    chain = chain - chain.mean(axis=0) + box / 2
    w = rng.random((n_water, 1, 3)) * box + rng.normal(scale=0.6, size=(n_water, 3, 3))
    xs = np.stack([chain + rng.normal(scale=0.2, size=chain.shape) for _ in range(nframes)])
    xv = np.stack([(w + rng.normal(scale=0.2, size=(n_water, 1, 3))).reshape(-1, 3) for _ in range(nframes)])
    return xs, xv, np.repeat(H[None], nframes, axis=0)


def engine_kw(n_solute, n_water, **extra):
    kw = dict(solute_nmols=1, solute_natomspermol=n_solute, solvent_nmols=n_water, solvent_natomspermol=3,
              autocorrelation=False, precision="fp32", regime="atoms", max_frames_per_batch=4, atoms_schedule="balanced",
              solute_groups=[[i // 10] for i in range(n_solute)], solute_ngroups=(n_solute + 9) // 10, **OPT)
    kw.update(extra)
    return kw


def alone(cm, xs, xv, cells, **kw):
    eng = cm.Engine(**kw)
    eng.submit(xs, xv, cells)
    out = eng.raw_counts()
    eng.close()
    return out


@pytest.mark.parametrize("grid", [-1, 3], ids=["walk", "grid"])
def test_fused_batch_equals_each_system_alone(cm, orc, gpu_ready, grid):
    """Six systems of uneven size (60-400 solute atoms, 100-900 waters), 3-7
    frames each (one or two compute chunks), in two calls, one system sitting
    the second call out: counts per system equal an engine of its own, and the
    first system's equal the oracle's."""
    rng = np.random.default_rng(61)
    sizes = [(60, 100, 3), (400, 900, 7), (150, 300, 5), (90, 700, 6), (300, 200, 4), (220, 500, 7)]
    systems, engines, want = [], [], []
    for n_s, n_w, nf in sizes:
        xs, xv, cells = chain_system(rng, n_s, n_w, nf, 24.0 + n_w / 60.0)
        kw = engine_kw(n_s, n_w, atoms_grid=grid)
        systems.append((xs, xv, cells, nf))
        engines.append(cm.Engine(**kw))
        want.append(alone(cm, xs, xv, cells, **kw))

    def part(k, lo, hi):
        xs, xv, cells, nf = systems[k]
        hi = min(hi, nf)
        if hi <= lo:
            return None
        return (xs[lo:hi], xv[lo:hi], cells[lo:hi], np.arange(lo + 1, hi + 1))

    with cm.Batch(engines) as b:
        b.submit([part(k, 0, 4) for k in range(len(systems))])
        b.submit([None if k == 2 else part(k, 4, 8) for k in range(len(systems))])
        st = b.graph_stats()
    # the second round holds the three systems with more than four frames
    assert st["fused_rounds"] == 2 and st["fused_systems"] == 3
    # one launch per stage for all systems: a round is tens of launches, not tens per system
    assert st["stage_launches"] <= 2 * 40
    got = []
    for e in engines:
        got.append(e.raw_counts())
        e.close()
    # system 2 never got its frames 5..: its engine alone saw all 5, compare against the first 4
    xs, xv, cells, _ = systems[2]
    want[2] = alone(cm, xs[:4], xv[:4], cells[:4], **engine_kw(150, 300, atoms_grid=grid))
    for k in range(len(systems)):
        for key in KEYS:
            assert np.array_equal(got[k][key], want[k][key]), (k, key)
    xs, xv, cells, nf = systems[0]
    kw = engine_kw(60, 100)
    ref = orc.run(ms=1, aps=60, mv=100, apv=3, solute_xyz=xs, solvent_xyz=xv, cells=cells,
                  frame_ids=list(range(1, nf + 1)), backend="cells", autocorrelation=False,
                  solute_groups=kw["solute_groups"], solute_ngroups=kw["solute_ngroups"], **OPT)
    for key in KEYS:
        assert np.array_equal(np.asarray(got[0][key]).ravel(), np.asarray(ref[key]).ravel()), key


@pytest.mark.parametrize("grid", [-1, 3], ids=["walk", "grid"])
def test_fused_and_streams_modes_agree(cm, gpu_ready, grid):
    """The same systems through a fused batch and a per-system-streams batch,
    resident frames, three rounds, the systems' evaluation schedules differing
    (a stage then takes one launch per kernel): identical counts."""
    import torch

    rng = np.random.default_rng(62)
    specs = [(80, 150, 4), (250, 600, 4), (120, 400, 4)]
    data = [chain_system(rng, n_s, n_w, nf, 26.0) for n_s, n_w, nf in specs]
    dev = [(torch.from_numpy(xs.astype(np.float32)).cuda(), torch.from_numpy(xv.astype(np.float32)).cuda(), cells)
           for xs, xv, cells in data]
    out = {}
    for mode in ("fused", "streams"):
        engines = [cm.Engine(**engine_kw(n_s, n_w, atoms_grid=grid, atoms_schedule=("cell", "balanced")[k % 2]))
                   for k, (n_s, n_w, _) in enumerate(specs)]
        with cm.Batch(engines, mode=mode) as b:
            for _ in range(3):
                b.submit(dev)
            st = b.graph_stats()
        assert (st["fused_rounds"] == 3) == (mode == "fused")
        out[mode] = [e.raw_counts() for e in engines]
        for e in engines:
            e.close()
    for k in range(len(specs)):
        for key in KEYS:
            assert np.array_equal(out["fused"][k][key], out["streams"][k][key]), (k, key)


def test_unfusable_round_falls_back(cm, gpu_ready):
    """A molecule-layout system in the batch: the round runs per-system
    streams, with the same counts as each engine alone."""
    rng = np.random.default_rng(63)
    xs, xv, cells = chain_system(rng, 100, 300, 3, 25.0)
    kw_a = engine_kw(100, 300)
    ms, aps = 40, 4
    ps = rng.random((ms, 1, 3)) * 25.0 + rng.normal(scale=0.8, size=(ms, aps, 3))
    xs_p = np.stack([ps.reshape(-1, 3) + rng.normal(scale=0.2, size=(ms * aps, 3)) for _ in range(3)])
    kw_p = dict(solute_nmols=ms, solute_natomspermol=aps, solvent_nmols=ms, solvent_natomspermol=aps,
                autocorrelation=True, precision="fp32", regime="pairs", max_frames_per_batch=4, **OPT)
    want = [alone(cm, xs, xv, cells, **kw_a), alone(cm, xs_p, None, cells, **kw_p)]
    engines = [cm.Engine(**kw_a), cm.Engine(**kw_p)]
    with cm.Batch(engines) as b:
        b.submit([(xs, xv, cells), (xs_p, None, cells)])
        st = b.graph_stats()
    assert st["fused_rounds"] == 0 and st["graph_launches"] == 1
    for k, e in enumerate(engines):
        got = e.raw_counts()
        e.close()
        for key in KEYS:
            if k == 1 and key.startswith("solvent"):
                continue
            assert np.array_equal(got[key], want[k][key]), (k, key)
