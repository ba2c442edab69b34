"""Request server (continuous batching) through the C ABI: every request's
counts are the same alone and in the mix, admission follows the device-memory
budget, and cancelled or oversized requests end in their own states."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
        "solvent_group_random")


def system(rng, L, ms, aps, mv, apv, nframes, self_mode):
    H = np.diag([L, L * 1.05, L * 0.97])

    def mols(n, apm):
        c = rng.random((n, 1, 3)) @ H.T
        return (c + rng.normal(scale=0.8, size=(n, apm, 3))).reshape(-1, 3)

    xs0 = mols(ms, aps)
    xv0 = None if self_mode else mols(mv, apv)
    xs = np.stack([xs0 + rng.normal(scale=0.2, size=xs0.shape) for _ in range(nframes)])
    xv = None if self_mode else np.stack([xv0 + rng.normal(scale=0.2, size=xv0.shape) for _ in range(nframes)])
    return xs, xv, np.repeat(H[None], nframes, axis=0)


def cm_setbin(d, step):
    """nbins of a cutoff: max(1, ceil(d / step)), as the reference's setbin."""
    return max(1, int(math.ceil(d / step)))


def requests():
    rng = np.random.default_rng(99)
    out = []
    specs = [  # (L, ms, aps, mv, apv, nframes, self, cutoff, precision)
        (30.0, 300, 3, 300, 3, 7, True, 8.0, "fp32"),
        (26.0, 20, 5, 400, 3, 5, False, 7.0, "fp32"),
        (40.0, 600, 14, 600, 14, 3, True, 10.0, "fp32"),
        (24.0, 1, 60, 500, 3, 9, False, 9.0, "fp32"),       # ATOMS layout (60-atom solute)
        (28.0, 250, 4, 250, 4, 6, True, 6.5, "fp64"),
        (22.0, 15, 3, 300, 3, 40, False, 8.0, "fp32"),      # many frames: several turns
    ]
    for L, ms, aps, mv, apv, nf, self_mode, cut, prec in specs:
        xs, xv, cells = system(rng, L, ms, aps, mv, apv, nf, self_mode)
        kw = dict(solute_nmols=ms, solute_natomspermol=aps, solvent_nmols=mv, solvent_natomspermol=apv,
                  autocorrelation=self_mode, irefatom=1, cutoff=cut, binstep=0.02, dbulk=cut, usecutoff=False,
                  nbins=cm_setbin(cut, 0.02), n_random_samples=4, seed=7, precision=prec)
        out.append((xs, xv, cells, kw))
    return out


def alone(cm, xs, xv, cells, kw):
    eng = cm.Engine(**kw)
    eng.submit(xs, xv, cells)
    r = eng.raw_counts()
    eng.close()
    return r


def test_mix_equals_alone(cm, gpu_ready):
    reqs = requests()
    ref = [alone(cm, *r) for r in reqs]
    with cm.Server(max_active=3, frames_per_turn=4) as srv:
        ids = [srv.submit(xs, xv, cells, **kw) for xs, xv, cells, kw in reqs]
        infos = [srv.wait(i, timeout=120) for i in ids]
        bad = []
        for rid, info in zip(ids, infos):
            if info["state"] != "done":
                try:
                    srv.counts(rid)
                except Exception as e:  # the request's own error message
                    bad.append((rid, info["state"], str(e)))
        assert not bad, bad
        for rid, r in zip(ids, ref):
            got = srv.raw_counts(rid)
            for k in KEYS:
                assert np.array_equal(got[k], r[k]), (rid, k)
        w = srv.counts(ids[0])
        assert w["frames"] == reqs[0][0].shape[0]
        for rid in ids:
            srv.release(rid)
        p = cm.latency_percentiles(infos)
        assert p["p50"] is not None and p["p99"] >= p["p50"]


def test_budget_admission_serialises_requests(cm, gpu_ready):
    """With a budget that holds one request at a time, each request is
    admitted only after the previous one has finished."""
    reqs = [requests()[2]] * 3   # three requests of one size
    probe = cm.Engine(max_frames_per_batch=2, **reqs[0][3])   # the server's handles stage frames_per_turn frames
    probe.submit(*reqs[0][:3])
    probe.synchronize()
    big = probe.device_bytes()
    probe.close()
    with cm.Server(hbm_budget_bytes=int(big * 1.3), frames_per_turn=2) as srv:
        ids = [srv.submit(xs, xv, cells, **kw) for xs, xv, cells, kw in reqs]
        infos = [srv.wait(i, timeout=120) for i in ids]
        assert all(i["state"] == "done" for i in infos), infos
        spans = sorted((i["t_admit"], i["t_done"]) for i in infos)
        for (a0, d0), (a1, d1) in zip(spans, spans[1:]):
            assert a1 >= d0 - 1e-6


def test_cancel_and_oversize(cm, gpu_ready):
    reqs = requests()
    with cm.Server(max_active=1, hbm_budget_bytes=64 << 20, frames_per_turn=1) as srv:
        first = srv.submit(*reqs[5][:3], **reqs[5][3])
        queued = srv.submit(*reqs[0][:3], **reqs[0][3])
        srv.cancel(queued)
        assert srv.wait(queued, timeout=60)["state"] == "cancelled"
        assert srv.wait(first, timeout=120)["state"] == "done"
        # a system far beyond the budget cannot run at all
        xs, xv, cells, kw = reqs[2]
        kw = dict(kw, hbm_budget_bytes=0)
        big = np.concatenate([xs] * 100, axis=1)   # 60,000 molecules: far above 64 MiB
        kw.update(solute_nmols=kw["solute_nmols"] * 100, solvent_nmols=kw["solvent_nmols"] * 100)
        rid = srv.submit(big, None, cells, **kw)
        info = srv.wait(rid, timeout=120)
        assert info["state"] == "failed"
        with pytest.raises(MemoryError):
            srv.counts(rid)


def test_handles_with_different_shared_memory_interleave(cm, gpu_ready):
    """Kernel shared-memory limits are process-wide: a handle planned later
    with smaller histograms must not break an earlier handle's launches."""
    reqs = requests()
    big, small = reqs[3], reqs[0]          # 65 histogram rows vs 5
    e1 = cm.Engine(**big[3])
    nf = big[0].shape[0]
    e1.submit(big[0][:4], big[1][:4], big[2][:4], frame_ids=np.arange(1, 5))
    e2 = cm.Engine(**small[3])
    e2.submit(*small[:3])
    e1.submit(big[0][4:], big[1][4:], big[2][4:], frame_ids=np.arange(5, nf + 1))
    got = e1.raw_counts()
    e1.close()
    e2.close()
    ref = alone(cm, *big)
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k


def test_closed_engines_return_memory_to_the_block_cache(cm):
    """A closed engine's device and pinned blocks go to the process-wide cache
    (freeing them would wait for every stream of the device); an engine of the
    same system opened next takes them back, and its counts are unchanged on
    the reused (not zeroed) memory."""
    xs, xv, cells, kw = requests()[3]
    first = alone(cm, xs, xv, cells, kw)
    before = cm.memory_cache(0)
    assert before["device_bytes"] > 0 and before["host_bytes"] > 0
    again = alone(cm, xs, xv, cells, kw)
    after = cm.memory_cache(0)
    assert after["device_bytes"] <= before["device_bytes"]
    for k in KEYS:
        assert np.array_equal(first[k], again[k]), k
    released = cm.memory_cache(0, release=True)
    assert released["device_bytes"] == 0 and released["host_bytes"] == 0
