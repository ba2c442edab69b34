#!/usr/bin/env python
"""MDDF throughput on the config-3 workload (self-MDDF in a triclinic cell).

Workload: 10,000 rigid 14-atom molecules (140,000 atoms) in a triclinic cell
a = b = c = 110 A, gamma = 60 degrees, 500 frames of sigma = 0.4 A jitter stored
as FP32, cutoff 10 A, binstep 0.02 A, 5 random-insertion samples per frame,
per-atom groups; seeded synthetic data (no dataset).  One step = all 500
frames through the engine.

  value   frames/s with the frames resident in HBM (FP32 search + FP64 guard)
  e2e     the same through the C ABI from pinned host memory, host-to-device
          copies and the read-out of the counts inside the timed region
  plain_fp64  the plain FP64 engine path on the same frames
  roofline    the real-pass kernel (FP32-issue bound; algorithmic flops =
              8 per atom pair within the cutoff) against the FP32 throughput
              measured on this GPU, plus its HBM figure; the guard kernel's
              FP64 re-evaluations are timed apart (kernel class "guard")
  cpu_baseline  the CPU restatement of the reference's per-frame path (oracle,
              all host threads) on a bounded sample of the frames

--workload c1 | c2-water | c2-cosolvent | c4 prints the frames/s of that
configuration's system (ATOMS layout) instead of the headline line;
--workload grid3d times grid3D's grid search on a 1,463-atom protein (the
NAMD test fixture) against the CPU restatement on a sample of the points.

--impl reference times that CPU path alone (the reference itself is Julia
and cannot run here).  Multi-GPU runs are independent replicas (the path
shards by frames with no exchange), launched one rank per GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NFRAMES = 500
NMOLS = 10000
APM = 14
CUTOFF = 10.0
BINSTEP = 0.02
NRAND = 5
SEED = 20261203 + 3
METRIC = "MDDF frames/s (config 3, batched FP32 + FP64 guard)"

# serving (config 5): requests carved from one large c3-density system, see c5_bank
SERVE_SEED = 20261203 + 5
C5_REQUESTS = 2000           # the configuration's request count (--workload c5)
C5_MAX_FRAMES = 200          # frames per request uniform in [1, 200]
C5_ATOMS = (5000, 500000)    # atoms per request log-uniform in this range
C5_BANK_MOLS = 36000         # 504,000 atoms: every request size is a part of this system
SERVE_REQUESTS = 250         # requests of the serving leg of the default bench line
SERVE_RATES = (1.0, 1.5, 2.0)  # arrival rates, multiples of the serial FP32 service rate
SERVE_MAX_ACTIVE = 2           # requests on the device at once (2 gave the highest aggregate rate of 2, 3, 4, 8 and 32)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="engine", choices=["engine", "reference"])
    p.add_argument("--frames", type=int, default=NFRAMES)
    p.add_argument("--cpu-frames", type=int, default=0, help="CPU-baseline sample size (0: one frame per host thread)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--serve-max-active", type=int, default=SERVE_MAX_ACTIVE,
                   help="serving: requests on the device at once (--workload c5 and the serving leg)")
    p.add_argument("--serve-requests", type=int, default=0, help="--workload c5: requests (0 = the configuration's 2,000)")
    p.add_argument("--serve-rates", default="", help="--workload c5: comma-separated arrival rates (x serial FP32)")
    p.add_argument("--atoms-grid", type=int, default=0,
                   help="ATOMS layout, one solute molecule: fine cells per search-cell axis of the candidate grid "
                        "(0 = engine default, -1 = stencil walk; speed only)")
    p.add_argument("--real-pass", default="auto", choices=["auto", "warp", "tile"],
                   help="FP32 real-pass schedule (speed only): per-molecule warps or home-cell tiles")
    p.add_argument("--workload", default="c3", choices=["c3", "c1", "c2-water", "c2-cosolvent", "c4", "c4-batch", "c5", "grid3d"],
                   help="c3 (default): the headline line; the others: frames/s of that configuration's system "
                        "(ATOMS layout) on device-resident frames")
    return p.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group(backend="gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(world, v):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(nframes):
    import __graft_entry__ as entry

    entry.load_package()
    syn = __import__("importlib").import_module(entry.PKG_NAME + ".synth")
    s = syn.config3(seed=SEED, nmols=NMOLS, nframes=nframes)
    xs, _, cells = s.frames(nframes)
    return xs.astype(np.float32), cells


def config_dict(nframes, extra=None):
    d = {
        "workload": "c3: self-MDDF, 10,000 rigid 14-atom molecules (140,000 atoms), triclinic a=b=c=110 A "
                    "gamma=60, FP32 frames, cutoff 10 A, binstep 0.02, 5 random samples/frame, per-atom groups",
        "frames_per_step": nframes,
        "atoms": NMOLS * APM,
        "cutoff": CUTOFF,
        "n_random_samples": NRAND,
        "precision": "fp32 search, fp64 guard band",
        "l2": "inputs are %.0f MB per step (L2 is 129 MB)" % (nframes * NMOLS * APM * 12 / 1e6),
        "seed": SEED,
    }
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        load = [v for v in sm if mx and v > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def c5_bank(syn, device, nframes=C5_MAX_FRAMES):
    """Frames of every config-5 request, resident on the device, from one
    large system at c3 density: 36,000 rigid 14-atom molecules (504,000 atoms)
    in a triclinic cell H (a = b = c, gamma = 60), uniform positions, random
    orientations, each frame rigid molecule translations of sigma = 0.4 A.
    The molecules are ordered by the largest fractional coordinate of their
    centroid, so the molecules whose centroids lie in the cell s H (s <= 1,
    the same shape) are a prefix: a request of n atoms takes s = (n / N)^(1/3),
    the prefix of molecules inside s H and the cell s H, i.e. a uniform c3-like
    system of about n atoms, and its frames are slices of the shared frames
    (frame stride N x 3), so no request copies coordinates."""
    import math

    import torch

    rng = np.random.default_rng(SERVE_SEED)
    dens = 10000 / (110.0**3 * math.sin(math.radians(60)))
    edge = (C5_BANK_MOLS / dens / math.sin(math.radians(60))) ** (1 / 3)
    H = syn.triclinic_cell(edge, edge, edge, 90.0, 90.0, 60.0)
    frac = rng.random((C5_BANK_MOLS, 3))
    order = np.argsort(frac.max(axis=1), kind="stable")
    frac = frac[order]
    x0 = syn.place_molecules(rng, syn.ball_template(rng, 14, 4.0), frac @ H.T).astype(np.float32)
    x0 = torch.from_numpy(x0.reshape(C5_BANK_MOLS, 14, 3)).to(device)
    gen = torch.Generator(device=device).manual_seed(SERVE_SEED)
    bank = torch.empty((nframes, C5_BANK_MOLS * 14, 3), dtype=torch.float32, device=device)
    for k in range(nframes):
        shift = torch.randn((C5_BANK_MOLS, 1, 3), generator=gen, device=device, dtype=torch.float32) * 0.4
        bank[k] = (x0 + shift).reshape(-1, 3)
    return bank, H, np.sort(frac.max(axis=1))


def c5_requests(H, mmax, nreq):
    """nreq requests: atoms log-uniform in C5_ATOMS, 1..C5_MAX_FRAMES frames,
    cutoff uniform in [8, 14] rounded to a multiple of 0.02 (Options accepts
    no other, src/Options.jl:167-172).  Each is (molecules, frames, cutoff, cell)."""
    rng = np.random.default_rng(SERVE_SEED + 1)
    reqs = []
    for _ in range(nreq):
        n = float(np.exp(rng.uniform(np.log(C5_ATOMS[0]), np.log(C5_ATOMS[1]))))
        sc = (n / (C5_BANK_MOLS * 14)) ** (1 / 3)
        nm = max(2, int(np.searchsorted(mmax, sc)))
        nf = int(rng.integers(1, C5_MAX_FRAMES + 1))
        cutoff = float(f"{round(rng.uniform(8.0, 14.0) / 0.02) * 0.02:.2f}")
        reqs.append((nm, nf, cutoff, H * sc))
    return reqs


def serving_leg(cm, device, nreq=SERVE_REQUESTS, rates=SERVE_RATES, fp64_sample=12, max_active=SERVE_MAX_ACTIVE,
                frames_per_turn=32):
    """Config-5 serving load: Poisson arrivals of c3-like self-MDDF requests
    (c5_bank, c5_requests) into the continuous-batching server (FP32 + guard)
    at several arrival rates, against the same requests run one at a time on
    the FP32 engine (the serial service rate, and the counts every request
    must reproduce) and a sample of them on the plain FP64 engine."""
    import hashlib

    import torch

    syn = __import__("importlib").import_module("complexmixtures_gb300.synth")
    dev = f"cuda:{device}"
    bank, H, mmax = c5_bank(syn, dev)
    reqs = c5_requests(H, mmax, nreq)
    frames_total = sum(nf for _, nf, _, _ in reqs)
    atoms = [nm * 14 for nm, _, _, _ in reqs]

    def kw(nm, cutoff, precision):
        return dict(solute_nmols=nm, solute_natomspermol=14, solvent_nmols=nm, solvent_natomspermol=14,
                    autocorrelation=True, irefatom=1, cutoff=cutoff, binstep=0.02, dbulk=cutoff, usecutoff=False,
                    nbins=cm.setbin(cutoff, 0.02), n_random_samples=5, seed=SERVE_SEED, precision=precision,
                    device=device)

    def frames(nm, nf):
        return bank[:nf, : nm * 14]

    def cells(cell, nf):
        return np.repeat(cell[None], nf, axis=0)

    def digest(raw):
        h = hashlib.sha256()
        for k in ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random"):
            h.update(np.ascontiguousarray(raw[k]).tobytes())
        return h.hexdigest()

    def serial(precision, which):
        out = {}
        torch.cuda.synchronize()
        t = time.perf_counter()
        for i in which:
            nm, nf, cutoff, cell = reqs[i]
            with cm.Engine(**kw(nm, cutoff, precision)) as eng:
                eng.submit(frames(nm, nf), None, cells(cell, nf))
                out[i] = digest(eng.raw_counts())
        return time.perf_counter() - t, out

    serial("fp32", range(min(8, nreq)))  # warm-up: module load, first allocations
    t32, ref = serial("fp32", range(nreq))
    rate32 = frames_total / t32
    sample = list(range(0, nreq, max(1, nreq // fp64_sample)))[:fp64_sample]
    t64, ref64 = serial("fp64", sample)
    sample_frames = sum(reqs[i][1] for i in sample)
    runs = []
    for mult in rates:
        rate = mult * nreq / t32
        gaps = np.random.default_rng(SERVE_SEED + 2).exponential(1.0 / rate, nreq)
        with cm.Server(device=device, frames_per_turn=frames_per_turn, max_active=max_active,
                       hbm_budget_bytes=96 << 30) as srv:
            ids = []
            t0 = time.perf_counter()
            due = t0
            for (nm, nf, cutoff, cell), g in zip(reqs, gaps):
                due += g
                while time.perf_counter() < due:
                    time.sleep(min(1e-4, max(0.0, due - time.perf_counter())))
                ids.append(srv.submit(frames(nm, nf), None, cells(cell, nf), **kw(nm, cutoff, "fp32")))
            infos = [srv.wait(r, timeout=1800) for r in ids]
            span = max(x["t_done"] for x in infos) - min(x["t_submit"] for x in infos)
            same = all(x["state"] == "done" and digest(srv.raw_counts(r)) == ref[k]
                       for k, (r, x) in enumerate(zip(ids, infos)))
        pct = cm.latency_percentiles(infos)
        runs.append({"arrival_rate_x_serial": mult, "arrival_rate_per_s": rate, "p50_ms": pct["p50"],
                     "p99_ms": pct["p99"], "frames_per_s": frames_total / span,
                     "failed": sum(1 for x in infos if x["state"] != "done"),
                     "counts_identical_to_serial": bool(same)})
    best = max(runs, key=lambda r: r["frames_per_s"])
    return {
        "workload": f"{nreq} Poisson-arrival self-MDDF requests, c3-like (14-atom molecules at c3 density, "
                    f"triclinic gamma=60), atoms log-uniform in [{C5_ATOMS[0]:,}, {C5_ATOMS[1]:,}] "
                    f"(drawn {min(atoms):,}-{max(atoms):,}), 1-{C5_MAX_FRAMES} frames each, cutoff U[8,14] "
                    f"rounded to 0.02, 5 random samples; frames resident on the device",
        "requests": nreq, "frames": frames_total,
        "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"], "frames_per_s": best["frames_per_s"],
        "serial_fp32_frames_per_s": rate32,
        "serial_fp64_frames_per_s": sample_frames / t64,
        "serial_fp64_sample": f"{len(sample)} of the requests ({sample_frames} frames)",
        "fp64_sample_counts_identical": all(ref64[i] == ref[i] for i in sample),
        "arrival_sweep": runs,
        "failed": sum(r["failed"] for r in runs),
        "counts_identical_to_serial": all(r["counts_identical_to_serial"] for r in runs),
    }


def c5_workload(args, local):
    """Config 5 at its stated load: 2,000 requests (serving_leg)."""
    import torch

    import __graft_entry__ as entry

    cm = entry.load_package()
    torch.cuda.set_device(local)
    rates = tuple(float(x) for x in args.serve_rates.split(",")) if args.serve_rates else SERVE_RATES
    out = serving_leg(cm, local, nreq=args.serve_requests or C5_REQUESTS, fp64_sample=20, rates=rates,
                      max_active=args.serve_max_active)
    out["max_active"] = args.serve_max_active
    out.update(metric="MDDF frames/s and request latency (config 5 serving load)", unit="frames/s",
               value=out["frames_per_s"], data="synthetic (seeded generator of the configuration)")
    print(json.dumps(out), flush=True)


C4_FRAMES = 50              # frames per config-4 system


def batched_c4_leg(cm, device):
    """Config-4 load: 64 independent systems of uneven size (2,000-200,000
    atoms, 5 % chain + water) run one at a time; as one batch whose kernels
    of all systems are one CUDA graph launch per staging round; and submitted
    together to the request server, which runs them concurrently on the
    device.  The cell size comes from the autotuner on the median system."""
    import torch

    syn = __import__("importlib").import_module("complexmixtures_gb300.synth")
    sizes = syn.config4_sizes()
    systems = []
    for k, n in enumerate(sizes):
        sysm = syn.config4_system(int(n), 20261207 + k, nframes=C4_FRAMES)
        xs, xv, cells = sysm.frames(C4_FRAMES)
        aps = sysm.solute_natomspermol
        sv = sysm.solvents[0]
        kw = dict(solute_nmols=1, solute_natomspermol=aps, solvent_nmols=sv.nmols, solvent_natomspermol=3,
                  autocorrelation=False, irefatom=1, cutoff=10.0, binstep=0.02, dbulk=10.0, usecutoff=False, nbins=500,
                  n_random_samples=10, seed=sysm.seed, solute_groups=[[i // 10] for i in range(aps)],
                  solute_ngroups=(aps + 9) // 10, precision="fp32", device=device)
        systems.append((xs, xv, cells, kw))
    med = int(np.argsort(sizes)[len(sizes) // 2])
    xs, xv, cells, kw = systems[med]
    tune = cm.autotune(xs[:8], xv[:8], cells[:8], **kw)
    pct = tune["cell_scale_pct"]
    sched = tune["atoms_schedule"]
    agrid = tune["atoms_grid"]
    frames_total = C4_FRAMES * len(systems)

    def serial():
        out = []
        torch.cuda.synchronize()
        t = time.perf_counter()
        for xs, xv, cells, kw in systems:
            eng = cm.Engine(cell_scale_pct=pct, atoms_schedule=sched, atoms_grid=agrid, **kw)
            eng.submit(xs, xv, cells)
            out.append(eng.raw_counts())
            eng.close()
        return time.perf_counter() - t, out

    def graph_batch():
        # all 64 systems in one cm_batch: one CUDA graph launch per staging round
        torch.cuda.synchronize()
        t = time.perf_counter()
        engines = [cm.Engine(cell_scale_pct=pct, atoms_schedule=sched, atoms_grid=agrid, **kw) for xs, xv, cells, kw in systems]
        with cm.Batch(engines) as b:
            b.submit([(xs, xv, cells) for xs, xv, cells, kw in systems])
            gst = b.graph_stats()
        out = [e.raw_counts() for e in engines]
        for e in engines:
            e.close()
        return time.perf_counter() - t, out, gst

    def resident_batch(mode, steps=3):
        # the systems stay resident: engines and batch made once, frames on the
        # device, each step one cm_batch_submit of every system's frames
        dev = [(torch.as_tensor(xs, device=device), torch.as_tensor(xv, device=device), cells)
               for xs, xv, cells, kw in systems]
        engines = [cm.Engine(cell_scale_pct=pct, atoms_schedule=sched, atoms_grid=agrid, **kw) for xs, xv, cells, kw in systems]
        with cm.Batch(engines, mode=mode) as b:
            b.submit(dev)  # warm-up
            for e in engines:
                e.reset()
            g0 = b.graph_stats()
            torch.cuda.synchronize()
            t = time.perf_counter()
            for _ in range(steps):
                b.submit(dev)
            for e in engines:
                e.synchronize()
            dt = time.perf_counter() - t
            g1 = b.graph_stats()
        out = [e.raw_counts() for e in engines]
        for e in engines:
            e.close()
        per = {k: (g1[k] - g0[k]) / steps for k in ("graph_launches", "fused_rounds", "stage_launches")}
        return dt / steps, out, per

    serial()  # warm-up
    ts, ref = serial()
    graph_batch()  # warm-up
    tg, gout, gst = graph_batch()
    same_graph = all(all(np.array_equal(gout[i][k], ref[i][k]) for k in ("md", "md_random", "solute_group"))
                     for i in range(len(systems)))
    tr, rout, rper = resident_batch("fused")
    # three steps of the same frames: each count is three times the one-pass count
    same_resident = all(all(np.array_equal(rout[i][k], 3 * ref[i][k]) for k in ("md", "md_random", "solute_group"))
                        for i in range(len(systems)))
    trs, rsout, rsper = resident_batch("streams")
    same_streams = all(all(np.array_equal(rsout[i][k], 3 * ref[i][k]) for k in ("md", "md_random", "solute_group"))
                       for i in range(len(systems)))
    with cm.Server(device=device, frames_per_turn=C4_FRAMES) as srv:
        t0 = time.perf_counter()
        ids = [srv.submit(xs, xv, cells, cell_scale_pct=pct, atoms_schedule=sched, atoms_grid=agrid, **kw) for xs, xv, cells, kw in systems]
        infos = [srv.wait(r, timeout=600) for r in ids]
        tb = time.perf_counter() - t0
        same = all(all(np.array_equal(srv.raw_counts(r)[k], ref[i][k]) for k in ("md", "md_random", "solute_group"))
                   for i, r in enumerate(ids))
    pct_lat = cm.latency_percentiles(infos)
    return {
        "workload": f"64 systems, atoms log-uniform in [2,000, 200,000] (5 % chain, rest 3-site water, "
                    f"0.1 atoms/A^3), {C4_FRAMES} FP32 frames each, cutoff 10 A, 10 random samples, groups of 10",
        "frames": frames_total,
        "serial_frames_per_s": frames_total / ts,
        "batched_frames_per_s": frames_total / tb,
        "graph_batch_frames_per_s": frames_total / tg,
        "graph_batch_launches": gst["graph_launches"],
        "graph_batch_counts_identical_to_serial": bool(same_graph),
        "graph_batch_resident_frames_per_s": frames_total / tr,
        "graph_batch_resident_counts_identical_to_serial": bool(same_resident),
        "graph_batch_resident_launches_per_step": rper,
        "graph_batch_resident_streams_frames_per_s": frames_total / trs,
        "graph_batch_resident_streams_counts_identical_to_serial": bool(same_streams),
        "graph_batch_resident_streams_launches_per_step": rsper,
        "p50_ms": pct_lat["p50"], "p99_ms": pct_lat["p99"],
        "cell_scale_pct": pct, "atoms_schedule": sched, "atoms_grid": agrid,
        "autotune_ms_per_frame": {f'{c["cell_scale_pct"]}/{c["atoms_schedule"]}/grid{c["atoms_grid"]}':
                                  round(c["ms_per_frame"], 4) for c in tune["candidates"]},
        "failed": sum(1 for x in infos if x["state"] != "done"),
        "counts_identical_to_serial": bool(same),
    }


def cpu_baseline(xs, cells, nframes_sample):
    """The oracle (CPU restatement of the reference's path), all host threads."""
    import __graft_entry__ as entry

    orc = entry.load_oracle()
    threads = os.cpu_count() or 1
    n = nframes_sample or max(4, min(threads, 16))
    n = min(n, xs.shape[0])
    t = time.perf_counter()
    out = orc.run(ms=NMOLS, aps=APM, mv=NMOLS, apv=APM, autocorrelation=True, irefatom=1, cutoff=CUTOFF,
                  binstep=BINSTEP, dbulk=CUTOFF, usecutoff=False, nbins=500, n_random_samples=NRAND, seed=SEED,
                  solute_xyz=xs[:n].astype(np.float64), solvent_xyz=None, cells=cells[:n],
                  frame_ids=np.arange(1, n + 1), nthreads=threads)
    dt = time.perf_counter() - t
    out["nframes"] = n
    return {"value": n / dt, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"first {n} of {xs.shape[0]} frames, one frame per thread (oracle/cm_oracle.c, cells backend)",
            "seconds": dt}, out


def run_reference(args, world, rank):
    """The reference arm: the CPU path of the reference (its restatement,
    kind "port"), timed on this machine's host cores."""
    if rank != 0:
        return
    xs, cells = workload(max(16, args.cpu_frames or 16))
    threads = os.cpu_count() or 1
    n = args.cpu_frames or max(4, min(threads, 16))
    times = []
    for i in range(args.warmup + args.steps):
        cb, _ = cpu_baseline(xs, cells, n)
        if i >= args.warmup:
            times.append(cb["seconds"])
    T = sum(times)
    v = args.steps * n / T
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * T / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, config-3 shapes)",
        "config": config_dict(n, {"step": f"{n} frames (bounded sample of the 500-frame workload)"}),
        "cpu_baseline": {"value": v, "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"{n} frames per step, one per thread"},
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Julia (not installed); its per-frame path is timed through the C restatement",
    }
    print(json.dumps(line), flush=True)


def other_workload(args, local):
    """Frames/s of one ATOMS-layout configuration (bench --workload), or the
    config-4 load of 64 systems (c4-batch)."""
    import torch

    import __graft_entry__ as entry

    cm = entry.load_package()
    torch.cuda.set_device(local)
    if args.workload == "c4-batch":
        out = batched_c4_leg(cm, local)
        out.update(metric="MDDF frames/s (config 4, 64 systems)", unit="frames/s",
                   value=out["graph_batch_resident_frames_per_s"])
        print(json.dumps(out), flush=True)
        return
    print(json.dumps(atoms_leg(cm, local, args.workload, args.steps, args.warmup, atoms_grid=args.atoms_grid)),
          flush=True)


_SYNTH_CACHE = {}


def atoms_leg(cm, local, workload, steps, warmup, atoms_grid=0):
    """Frames/s of one ATOMS-layout configuration (FP32 + guard, frames in
    HBM), with the per-class kernel times, the guard statistics and the plain
    FP64 path on the same frames; the config-4 case is its median system
    (43,000 atoms)."""
    import torch

    syn = __import__("importlib").import_module("complexmixtures_gb300.synth")
    nframes, solvent = 10, 0
    if workload == "c1":
        sysm = syn.config1()
    elif workload.startswith("c2"):
        if "c2" not in _SYNTH_CACHE:
            _SYNTH_CACHE["c2"] = syn.config2()
        sysm, nframes = _SYNTH_CACHE["c2"], 4
        solvent = 0 if workload == "c2-water" else 1
    else:
        sysm = syn.config4_system(43000, 20261207 + 43000, nframes=16)
        nframes = 16
    xs, xv, cells = sysm.frames(nframes, solvent=solvent)
    sv = sysm.solvents[solvent]
    aps = sysm.solute_natomspermol
    kw = dict(solute_nmols=sysm.solute_nmols, solute_natomspermol=aps, solvent_nmols=sv.nmols,
              solvent_natomspermol=sv.natomspermol, autocorrelation=False, irefatom=1, cutoff=sysm.cutoff,
              binstep=sysm.binstep, dbulk=sysm.cutoff, usecutoff=False, nbins=cm.setbin(sysm.cutoff, sysm.binstep),
              n_random_samples=sysm.n_random_samples, seed=sysm.seed, device=local,
              solute_groups=[[i // 10] for i in range(aps)], solute_ngroups=(aps + 9) // 10)
    xd = torch.from_numpy(xs).to(f"cuda:{local}")
    vd = torch.from_numpy(xv).to(f"cuda:{local}")
    ids = np.arange(1, nframes + 1)
    eng = cm.Engine(precision="fp32", kernel_timing=True, atoms_grid=atoms_grid, **kw)
    stream = torch.cuda.ExternalStream(eng.stream_ptr(), device=f"cuda:{local}")
    for _ in range(max(warmup, 1)):
        eng.submit(xd, vd, cells, frame_ids=ids)
    eng.synchronize()
    eng.reset()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        eng.submit(xd, vd, cells, frame_ids=ids)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    kt = eng.kernel_times()
    st = eng.stats()
    raw32 = eng.raw_counts()
    eng.close()
    frames = steps * nframes
    # the plain FP64 path on the same frames: its frames/s and the count comparison
    eng64 = cm.Engine(precision="fp64", **kw)
    s64 = torch.cuda.ExternalStream(eng64.stream_ptr(), device=f"cuda:{local}")
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s64)
    for _ in range(steps):
        eng64.submit(xd, vd, cells, frame_ids=ids)
    b.record(s64)
    b.synchronize()
    ms64 = a.elapsed_time(b)
    raw64 = eng64.raw_counts()
    eng64.close()
    hits = st["hits_real"] + st["hits_random"]
    return {
        "workload": workload, "metric": "MDDF frames/s", "value": frames / (ms / 1e3), "unit": "frames/s",
        "steps": steps, "warmup": warmup, "frames_per_step": nframes,
        "atoms": {"solute": int(sysm.solute_nmols * aps), "solvent": int(sv.nmols * sv.natomspermol)},
        "layout": "ATOMS" if st["regime"] == 2 else "PAIRS", "atoms_grid": atoms_grid,
        "kernel_ms_per_frame": {k: v[0] / frames for k, v in kt.items()},
        "guard": {"band_A": st["guard_band"], "reevaluations": st["guard_reevaluations"],
                  "rate_per_record": st["guard_reevaluations"] / hits if hits else 0.0,
                  "max_fp32_error_A": st["max_guard_error"]},
        "per_frame": {"molecule_pairs_evaluated": st["molecule_pairs_evaluated"] / frames,
                      "atom_pairs_evaluated": st["atom_pairs_evaluated"] / frames,
                      "hits": hits / frames},
        "plain_fp64": {"value": frames / (ms64 / 1e3), "unit": "frames/s",
                       "counts_identical_to_fp32_guard": all(np.array_equal(raw32[k], raw64[k]) for k in raw32)},
        "precision": "fp32 search, fp64 guard band", "data": "synthetic (seeded generator of the configuration)",
    }


def grid3d_workload(args, local):
    """grid3D's grid search (cm_grid3d) around the 1,463-atom protein of the
    NAMD test fixture, dmin 1.5, dmax 5, step 0.5 (about 10^6 points), from
    the MDDF of the protein against TMAO; the CPU restatement (numpy, one
    thread) is timed on a sample of the points and scaled per point."""
    import __graft_entry__ as entry

    cm = entry.load_package()
    g = np.load(os.path.join(ROOT, "tests", "golden", "namd_frames.npz"))
    cells = np.array([np.diag([c[0], c[2], c[5]]) for c in g["cells"]])
    protein = cm.AtomSelection.from_indices(list(range(1, 1464)), nmols=1)
    tmao = cm.AtomSelection.from_indices(list(range(1479, 4013)), natomspermol=14)
    tr = cm.ArrayTrajectory(protein, tmao, solute_frames=g["protein"].astype(np.float64),
                            solvent_frames=g["tmao"].astype(np.float64), cells=cells)
    R = cm.mddf(tr, cm.make_options(dbulk=10.0, n_random_samples=20, seed=4, silent=True), device=local)
    atoms = cm.Atoms(g["protein"][0].astype(np.float64))
    for _ in range(max(args.warmup, 1)):
        G = cm.grid3D(R, atoms, device=local)
    t = time.perf_counter()
    for _ in range(args.steps):
        G = cm.grid3D(R, atoms, device=local)
    dt = (time.perf_counter() - t) / args.steps
    npts = int(np.prod(G.n))
    orc = entry.load_oracle()
    idx = np.asarray(R.solute.indices)
    table = cm.grid3d.atom_contribution_table(R, "mddf")
    t = time.perf_counter()
    sample = orc.grid3d(atoms.xyz[idx - 1], (idx - idx[0]) % R.solute.natomspermol, table, R.d, dmin=1.5, dmax=5.0,
                        step=0.5, limit=20000)
    dc = time.perf_counter() - t
    print(json.dumps({
        "workload": "grid3d", "metric": "grid points/s", "value": npts / dt, "unit": "points/s",
        "points": npts, "kept": len(G), "ms_per_grid": dt * 1e3, "steps": args.steps,
        "api": "grid3D (cm_grid3d, host cell list and copies included)",
        "cpu_baseline": {"value": sample["evaluated"] / dc, "unit": "points/s", "cores": 1, "kind": "port",
                         "sample": f"first {sample['evaluated']} grid points (oracle/oracle.py grid3d, numpy)"},
    }), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "grid3d":
        if rank == 0:
            grid3d_workload(args, local)
        return
    if args.workload == "c5":
        if rank == 0:
            c5_workload(args, local)
        return
    if args.workload != "c3":
        if rank == 0:
            other_workload(args, local)
        return
    import torch

    import __graft_entry__ as entry

    cm = entry.load_package()
    torch.cuda.set_device(local)
    nf = args.frames
    xs, cells = workload(nf)
    ids = np.arange(1, nf + 1)
    xs_dev = torch.from_numpy(xs).to(f"cuda:{local}")
    xs_pin = torch.from_numpy(xs).pin_memory()

    def engine(precision, timing, chunk=nf):
        return cm.Engine(solute_nmols=NMOLS, solute_natomspermol=APM, solvent_nmols=NMOLS, solvent_natomspermol=APM,
                         autocorrelation=True, irefatom=1, cutoff=CUTOFF, binstep=BINSTEP, dbulk=CUTOFF,
                         usecutoff=False, nbins=500, n_random_samples=NRAND, seed=SEED, precision=precision,
                         device=local, max_frames_per_batch=chunk, kernel_timing=timing,
                         real_pass=args.real_pass)

    eng = engine("fp32", True)
    stream = torch.cuda.ExternalStream(eng.stream_ptr(), device=f"cuda:{local}")
    for _ in range(max(args.warmup, 3)):
        eng.submit(xs_dev, None, cells, frame_ids=ids)
    eng.synchronize()
    eng.reset()
    st0 = eng.stats()

    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        eng.submit(xs_dev, None, cells, frame_ids=ids)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    ms = allmax(world, ms)
    st = eng.stats()
    kt = eng.kernel_times()
    raw = eng.raw_counts()
    eng.close()
    value = world * args.steps * nf / (ms / 1e3)

    # end to end through the C ABI from pinned host memory, counts read back
    # host frames are staged in chunks of 50 so copies overlap compute
    eng2 = engine("fp32", False, chunk=min(50, nf))
    eng2.submit(xs_pin, None, cells, frame_ids=ids)
    eng2.counts()
    barrier(world)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        eng2.submit(xs_pin, None, cells, frame_ids=ids)
        counts = eng2.counts()
    e2e_s = allmax(world, time.perf_counter() - t)
    d2h = sum(v.nbytes for v in counts.values() if isinstance(v, np.ndarray))
    eng2.close()
    e2e = {"value": world * args.steps * nf / e2e_s, "unit": "frames/s",
           "h2d_bytes_per_step": int(xs.nbytes + cells.nbytes + 8 * nf * 2), "d2h_bytes_per_step": int(d2h),
           "api": "Engine.submit (cm_submit_frames, host memory) + Engine.counts (cm_read_counts)"}

    # plain FP64 path
    plain = None
    if not args.no_fp64:
        eng3 = engine("fp64", True)
        eng3.submit(xs_dev, None, cells, frame_ids=ids)
        eng3.synchronize()
        eng3.reset()
        s3 = torch.cuda.ExternalStream(eng3.stream_ptr(), device=f"cuda:{local}")
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s3)
        eng3.submit(xs_dev, None, cells, frame_ids=ids)
        b.record(s3)
        b.synchronize()
        ms64 = allmax(world, a.elapsed_time(b))
        kt64 = eng3.kernel_times()
        raw64 = eng3.raw_counts()
        eng3.close()
        same = all(np.array_equal(raw[k], raw64[k] * args.steps) for k in ("md", "md_random", "rdf", "rdf_random",
                                                                          "solute_group", "solute_group_random"))
        plain = {"value": world * nf / (ms64 / 1e3), "unit": "frames/s", "ms_per_step": ms64,
                 "real_kernel_ms_per_frame": kt64["real"][0] / nf,
                 "counts_identical_to_fp32_guard": bool(same)}

    # roofline of the dominant kernel: the real pass
    peak = cm._native.measure_fp32_peak(local)
    # the real pass runs one launch per compute chunk of up to 32 frames; its
    # time per frame is the class total over the frames of the timed steps
    frames_timed = args.steps * nf
    ms_real_frame = kt["real"][0] / frames_timed
    chunks = -(-nf // 32) * args.steps
    cpu = None
    W_real = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, out = cpu_baseline(xs, cells, args.cpu_frames)
        W_real = out["pairs_real"] / out["nframes"]
        cpu.pop("seconds", None)
    else:
        W_real = 7.13e7
    flops = 8.0 * W_real
    achieved = flops / (ms_real_frame * 1e-3) / 1e12
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    # algorithmic bytes of the real pass per frame: the FP32 molecule table
    # (centroid float4) and atom offsets (float4) it reads
    bytes_frame = 16.0 * NMOLS + 16.0 * NMOLS * APM
    # the self-MDDF real pass: home-cell tiles unless --real-pass warp
    tiled = args.real_pass != "warp"
    roofline = {
        "bound": "fp32",
        "kernel": ("k_pairs_tile32<14>" if tiled else "k_pairs_flat32<self, 14>") + " (one launch per chunk of 32 frames)",
        "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
        "peak_source": "FP32 FMA throughput measured by cm_measure_fp32_peak on this GPU (of measured)",
        "traffic": None,
        "work": f"8 flops x {W_real:.4g} atom pairs within the cutoff per frame, 32 frames per launch",
        "launch_ms": kt["real"][0] / chunks,
        "frames_per_launch": nf / (chunks / args.steps),
        "hbm": {"achieved_gbs": bytes_frame / (ms_real_frame * 1e-3) / 1e9, "peak_gbs": hbm_peak,
                "frac": bytes_frame / (ms_real_frame * 1e-3) / 1e9 / hbm_peak,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s"},
    }
    # DRAM bytes per launch from the committed ncu capture of this kernel on
    # this workload (first number of the file)
    traffic_file = os.path.join(ROOT, "profiles", "pairs_tile32_c3_traffic.txt" if tiled else "pairs_flat32_c3_traffic.txt")
    if os.path.exists(traffic_file):
        try:
            roofline["traffic"] = float(open(traffic_file).read().split()[0])
        except Exception:
            pass

    serving = batched = None
    atoms_configs = None
    if not args.no_serving and world == 1:
        serving = serving_leg(cm, local)
        batched = batched_c4_leg(cm, local)
        # the other configurations' systems (ATOMS layout), a few frames each
        atoms_configs = {w: atoms_leg(cm, local, w, steps=2, warmup=1) for w in ("c1", "c2-water", "c2-cosolvent", "c4")}

    launches = st["kernel_launches"] - st0["kernel_launches"]
    line = {
        "metric": METRIC, "value": value, "unit": "frames/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, config-3 shapes and distributions)",
        "config": config_dict(nf, {"parallelism": "replicas" if world > 1 else "single GPU",
                                   "real_pass": args.real_pass}),
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clk, "roofline": roofline, "cpu_baseline": cpu,
        "plain_fp64": plain,
        "fp32_guard_speedup_vs_plain_fp64": (value / world) / plain["value"] * world if plain else None,
        "pair_evaluations_per_s": st["atom_pairs_evaluated"] / (ms / 1e3) * world,
        "guard": {"reevaluations_per_frame": st["guard_reevaluations"] / max(1, st["frames"]),
                  "hits_per_frame": (st["hits_real"] + st["hits_random"]) / max(1, st["frames"]),
                  "max_fp32_error_A": st["max_guard_error"]},
        "kernel_ms_per_step": {k: v[0] / args.steps for k, v in kt.items()},
        "atoms_configs": atoms_configs,
        "serving": serving,
        "batched_c4": batched,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
