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
