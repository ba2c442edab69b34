"""Shared test helpers: build systems, run the oracle through the package's
host-side Result logic (frame selection, weights, finalisation)."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def frames_of(traj, frame_ids):
    """Read the wanted (1-based) frames of a trajectory sequentially."""
    xs, xv, cells = [], [], []
    want = set(frame_ids)
    traj.opentraj()
    traj.firstframe()
    for i in range(1, max(frame_ids) + 1):
        traj.nextframe()
        if i in want:
            xs.append(np.array(traj.x_solute, dtype=np.float64))
            xv.append(np.array(traj.x_solvent, dtype=np.float64))
            c = np.asarray(traj.getunitcell(), dtype=np.float64)
            cells.append(np.diag(c) if c.shape == (3,) else c)
    traj.closetraj()
    return np.stack(xs), np.stack(xv), np.stack(cells)


def system_kwargs(R, options, irefatom, coordination_number_only=False):
    """Keyword arguments shared by Engine(...) and oracle.run(...)."""
    solvent_sel = R.solute if R.autocorrelation else R.solvent
    sg = R.solute.solute_credit_table()
    vg = solvent_sel.solvent_credit_table()
    return dict(
        autocorrelation=R.autocorrelation, irefatom=irefatom, cutoff=options.cutoff, binstep=options.binstep,
        dbulk=options.dbulk, usecutoff=options.usecutoff, nbins=R.nbins, n_random_samples=options.n_random_samples,
        seed=options.seed, coordination_number_only=coordination_number_only,
        solute_groups=sg, solute_ngroups=R.solute.ngroups(), solvent_groups=vg, solvent_ngroups=solvent_sel.ngroups(),
    )


def oracle_mddf(cm, orc, traj, options, *, frame_weights=None, coordination_number_only=False, backend="brute",
                stop=False):
    """mddf() with the oracle computing the per-frame counts: the same frame
    selection, weight classes (folded in frame order, sum += w * n / 2) and
    finalisation as the package driver."""
    tmeta = cm.trajectory_metadata(traj, options)
    R = cm.new_result(traj, options, tmeta, frame_weights)
    fw = np.asarray(R.files[0].frame_weights)
    ids = [i for i in range(options.firstframe, tmeta.lastframe_read + 1, options.stride) if fw[i - 1] != 0.0]
    kw = system_kwargs(R, options, tmeta.irefatom, coordination_number_only)
    keys = ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
            "solvent_group_random")
    fields = ("md_count", "md_count_random", "rdf_count", "rdf_count_random", "solute_group_count",
              "solute_group_count_random", "solvent_group_count", "solvent_group_count_random")
    sums = {k: None for k in keys}
    vol = 0.0
    if ids and not stop:
        xs, xv, cells = frames_of(traj, ids)
        # runs of equal weight, in frame order
        runs = []
        for k, i in enumerate(ids):
            if runs and fw[runs[-1][-1][1] - 1] == fw[i - 1]:
                runs[-1].append((k, i))
            else:
                runs.append([(k, i)])
        for run in runs:
            sel = [k for k, _ in run]
            w = float(fw[run[0][1] - 1])
            out = orc.run(ms=R.solute.nmols, aps=R.solute.natomspermol, mv=R.solvent.nmols,
                          apv=R.solvent.natomspermol, solute_xyz=xs[sel],
                          solvent_xyz=None if R.autocorrelation else xv[sel], cells=cells[sel],
                          frame_ids=[i for _, i in run], backend=backend, **kw)
            for k in keys:
                v = out[k].astype(np.float64)
                inc = w * (v / 2.0)
                sums[k] = inc if sums[k] is None else sums[k] + inc
            for k in sel:
                vol += w * orc.cell_volume(cells[k])
    for k, f in zip(keys, fields):
        if sums[k] is not None:
            v = sums[k]
            if f.startswith("solvent_group") and R.autocorrelation:
                v = np.zeros_like(getattr(R, f))
            setattr(R, f, v.reshape(getattr(R, f).shape))
    R.volume.total = vol
    return cm.finalresults(R, options, coordination_number_only=coordination_number_only)


KEYS = ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
        "solvent_group_random")

TRICLINIC = np.array([[24.0, 12.0, 0.0], [0.0, 20.78460969082653, 0.0], [0.0, 0.0, 23.0]])
ORTHO = np.diag([23.0, 25.0, 24.0])


def make_system(rng, H, ms, aps, mv, apv, nframes, self_mode, spread=0.9):
    def mols(n, apm):
        c = rng.random((n, 1, 3)) @ H.T
        return (c + rng.normal(scale=spread, size=(n, apm, 3))).reshape(-1, 3)

    xs0 = mols(ms, aps)
    xv0 = None if self_mode else mols(mv, apv)
    xs = np.stack([xs0 + rng.normal(scale=0.15, size=xs0.shape) for _ in range(nframes)])
    xv = None if self_mode else np.stack([xv0 + rng.normal(scale=0.15, size=xv0.shape) for _ in range(nframes)])
    cells = np.repeat(H[None], nframes, axis=0)
    return xs, xv, cells


def compare(cm, orc, *, ms, aps, mv, apv, xs, xv, cells, self_mode, precision, regime, frame_ids=None, groups=None,
            backend="cells", dtype=np.float64, cell_scale_pct=0, atoms_schedule="auto", engine_kw=None, **opt):
    nf = xs.shape[0]
    frame_ids = list(range(1, nf + 1)) if frame_ids is None else frame_ids
    kw = dict(autocorrelation=self_mode, **opt)
    g = {}
    if groups == "custom":
        # overlapping custom groups: atom j in groups j % 3 and 3 (+ a group of
        # the first half of the atoms); solute side by local index
        gs = [[a % 3, 3] + ([4] if a < aps // 2 else []) for a in range(aps)]
        gv_rows = (lambda n, apm: [[j % 3, 3] + ([4] if (j % apm) < apm // 2 else []) for j in range(n)])
        gv = gv_rows(mv * apv, apv)
        g = dict(solute_groups=gs, solute_ngroups=5, solvent_groups=gv, solvent_ngroups=5)
    eng = cm.Engine(solute_nmols=ms, solute_natomspermol=aps, solvent_nmols=mv, solvent_natomspermol=apv,
                    precision=precision, regime=regime, max_frames_per_batch=2, cell_scale_pct=cell_scale_pct,
                    atoms_schedule=atoms_schedule, **kw, **(engine_kw or {}),
                    **g)
    eng.submit(xs.astype(dtype), None if self_mode else xv.astype(dtype), cells, frame_ids=frame_ids)
    got = eng.raw_counts()
    st = eng.stats()
    eng.close()
    ref = orc.run(ms=ms, aps=aps, mv=mv, apv=apv, solute_xyz=xs.astype(dtype).astype(np.float64),
                  solvent_xyz=None if self_mode else xv.astype(dtype).astype(np.float64), cells=cells,
                  frame_ids=frame_ids, backend=backend, **kw, **g)
    for k in KEYS:
        if self_mode and k.startswith("solvent"):
            continue
        assert np.array_equal(got[k], ref[k]), (k, np.nonzero(got[k] != ref[k]))
    return got, ref, st
