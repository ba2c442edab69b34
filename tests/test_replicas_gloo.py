"""Replicas path on CPU: two gloo ranks shard the frames, each computes its
counts, and the summed counts equal the single-process counts exactly.  The
per-rank compute here is the oracle (no GPU on this machine); on GPUs each
rank runs its own engine with the same sharding and reduction."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

KEYS = ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random")


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def system():
    rng = np.random.default_rng(3)
    L = 16.0
    H = np.diag([L, L, L])
    base = rng.random((30, 1, 3)) * L + rng.normal(scale=0.6, size=(30, 3, 3))
    frames = np.stack([base.reshape(-1, 3) + rng.normal(scale=0.1, size=(90, 3)) for _ in range(5)])
    kw = dict(ms=30, aps=3, mv=30, apv=3, autocorrelation=True, irefatom=1, cutoff=5.0, binstep=0.05, dbulk=5.0,
              usecutoff=False, nbins=100, n_random_samples=3, seed=4)
    return frames, np.repeat(H[None], 5, axis=0), kw


def rank_main(rank, world, port, q):
    import torch.distributed as dist

    import __graft_entry__ as entry

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cm = entry.load_package()
    from complexmixtures_gb300.replicas import allreduce_counts, frame_range

    orc = entry.load_oracle()
    frames, cells, kw = system()
    a, b = frame_range(len(frames), rank, world)
    part = orc.run(solute_xyz=frames[a:b], solvent_xyz=None, cells=cells[a:b], frame_ids=np.arange(a + 1, b + 1),
                   nthreads=1, **kw)
    total = allreduce_counts({k: part[k] for k in KEYS})
    if rank == 0:
        q.put({k: total[k] for k in KEYS})
    dist.barrier()
    dist.destroy_process_group()


def test_frame_range_covers_all():
    from importlib import import_module

    import __graft_entry__ as entry

    entry.load_package()
    fr = import_module("complexmixtures_gb300.replicas").frame_range
    for n in (0, 1, 5, 17):
        for w in (1, 2, 3, 8):
            got = [fr(n, r, w) for r in range(w)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(got[i][1] == got[i + 1][0] for i in range(w - 1))
            assert max(b - a for a, b in got) - min(b - a for a, b in got) <= 1
    with pytest.raises(ValueError):
        fr(5, 2, 2)


def test_two_gloo_ranks_sum_to_single_process(orc):
    frames, cells, kw = system()
    ref = orc.run(solute_xyz=frames, solvent_xyz=None, cells=cells, frame_ids=np.arange(1, len(frames) + 1),
                  nthreads=1, **kw)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k
