"""mddf / coordination_number drivers (src/mddf.jl:186-347, 539-585).

The reference reads frames one at a time and hands each to ``mddf_frame!`` on
a CPU thread.  Here frames are read in batches and handed to the GPU engine
(``Engine.submit``); the counts come back once at the end, then the unchanged
host-side finalisation runs (src/results.jl:311-469).
"""
from __future__ import annotations

import os
from typing import Optional

import numpy as np

from .engine import Engine
from .options import Options, TrajectoryFileOptions
from .results import Result, check_frame_weights, finalresults, isautocorrelation, setbin, sum_frame_weights
from .trajectory import ArrayTrajectory, NamdDCD, Trajectory, cell_matrix, make_trajectory, trajectory_metadata

STOP_FILE = "stop_complexmixtures"


def engine_for(R: Result, options: Options, irefatom: int, *, coordination_number_only: bool = False,
               precision: str = "fp32", regime: str = "auto", device: int = 0, max_frames_per_batch: int = 0,
               hbm_budget_bytes: int = 0) -> Engine:
    """Engine configured from a Result's selections and the run options."""
    solute_groups = R.solute.solute_credit_table()
    solvent_sel = R.solute if R.autocorrelation else R.solvent
    solvent_groups = solvent_sel.solvent_credit_table()
    return Engine(
        solute_nmols=R.solute.nmols,
        solute_natomspermol=R.solute.natomspermol,
        solvent_nmols=R.solvent.nmols,
        solvent_natomspermol=R.solvent.natomspermol,
        autocorrelation=R.autocorrelation,
        irefatom=irefatom,
        cutoff=options.cutoff,
        binstep=options.binstep,
        dbulk=options.dbulk,
        usecutoff=options.usecutoff,
        nbins=R.nbins,
        n_random_samples=options.n_random_samples,
        lcell=options.lcell,
        coordination_number_only=coordination_number_only,
        precision=precision,
        regime=regime,
        seed=options.seed,
        solute_groups=solute_groups,
        solute_ngroups=R.solute.ngroups(),
        solvent_groups=solvent_groups,
        solvent_ngroups=solvent_sel.ngroups(),
        device=device,
        max_frames_per_batch=max_frames_per_batch,
        hbm_budget_bytes=hbm_budget_bytes,
    )


def engine_stats_summary(st: dict) -> dict:
    """The engine's statistics of one run, reported with its Result (not saved
    with it): the FP32 search's guard band, how many minimum-distance records
    it sent to the exact FP64 rules (count and rate per record within the
    cutoff), and the largest FP32 distance error seen among them."""
    hits = st["hits_real"] + st["hits_random"]
    return {
        "frames": st["frames"],
        "atom_pairs_evaluated": st["atom_pairs_evaluated"],
        "records_within_cutoff": hits,
        "guard_reevaluations": st["guard_reevaluations"],
        "guard_rate": st["guard_reevaluations"] / hits if hits else 0.0,
        "max_fp32_error": st["max_guard_error"],
        "guard_band": st["guard_band"],
        "regime": "atoms" if st["regime"] == 2 else "pairs",
    }


def new_result(trajectory: Trajectory, options: Options, tmeta, frame_weights) -> Result:
    """Result constructor (src/results.jl:124-193)."""
    fw = check_frame_weights(frame_weights, options, tmeta.lastframe_read)
    return Result(
        nbins=setbin(options.cutoff, options.binstep),
        dbulk=options.dbulk,
        cutoff=options.cutoff,
        autocorrelation=isautocorrelation(trajectory.solute.indices, trajectory.solvent.indices),
        solute=trajectory.solute,
        solvent=trajectory.solvent,
        files=[
            TrajectoryFileOptions(
                filename=trajectory.filename,
                options=options,
                irefatom=tmeta.irefatom,
                lastframe_read=tmeta.lastframe_read,
                nframes_read=tmeta.nframes_read,
                frame_weights=[float(w) for w in fw],
            )
        ],
        weights=[1.0],
    )


def mddf(trajectory, solute=None, solvent=None, options: Optional[Options] = None, *, frame_weights=None,
         coordination_number_only: bool = False, low_memory: bool = False, trajectory_format: str = "",
         precision: str = "fp32", regime: str = "auto", device: int = 0, batch_frames: int = 64,
         finalize: str = "host", keep_engine: bool = False) -> Result:
    """Minimum-distance distribution function (src/mddf.jl:113-347).

    ``mddf(trajectory, options)`` with a Trajectory object, or
    ``mddf(filename, solute, solvent, options)`` / ``mddf(filename, solute,
    options)`` (self-MDDF) with a file name.  ``low_memory`` is accepted for
    signature compatibility; the GPU engine has a single memory layout.
    ``precision`` selects the FP32+guard ("fp32") or plain FP64 ("fp64") path;
    both give identical counts.  ``finalize="device"`` computes the
    normalisation, densities, MDDF, RDF and KB integrals on the GPU
    (cm_read_results) instead of the host restatement of finalresults!; both
    agree to 1e-12.  ``keep_engine=True`` leaves the engine open, with the
    run's accumulators on the device, as ``R.engine``: ``contributions`` and
    ``ResidueContributions`` then run on the GPU.  Close it with
    ``R.engine.close()``.
    """
    if finalize not in ("host", "device"):
        raise ValueError("finalize must be 'host' or 'device'")
    if isinstance(trajectory, str):
        if isinstance(solvent, Options) and options is None:
            options, solvent = solvent, None
        trajectory = make_trajectory(trajectory, solute, solvent, format=trajectory_format,
                                     lastframe=(options.lastframe if options else -1))
    elif isinstance(solute, Options) and options is None:
        options = solute
    options = options or Options()
    tmeta = trajectory_metadata(trajectory, options)
    R = new_result(trajectory, options, tmeta, frame_weights)
    fw = np.asarray(R.files[0].frame_weights)
    to_compute = [i for i in range(options.firstframe, tmeta.lastframe_read + 1, options.stride) if fw[i - 1] != 0.0]
    eng = engine_for(R, options, tmeta.irefatom, coordination_number_only=coordination_number_only,
                     precision=precision, regime=regime, device=device, max_frames_per_batch=batch_frames)
    ok = False
    try:
        _run_frames(eng, trajectory, to_compute, fw, batch_frames)
        if finalize == "device":
            res = eng.results(sum_frame_weights(R))
        else:
            c = eng.counts()
        stats = eng.stats()
        ok = True
    finally:
        if not (ok and keep_engine):
            eng.close()
    if keep_engine:
        R.engine = eng
    R.engine_stats = engine_stats_summary(stats)
    if finalize == "device":
        return _device_result(R, res, options, coordination_number_only)
    for k in ("md_count", "md_count_random", "rdf_count", "rdf_count_random", "solute_group_count",
              "solute_group_count_random", "solvent_group_count", "solvent_group_count_random"):
        setattr(R, k, c[k].copy())
    R.volume.total = c["volume_total"]
    return finalresults(R, options, coordination_number_only=coordination_number_only)


def _device_result(R: Result, res: dict, options: Options, coordination_number_only: bool) -> Result:
    """A Result filled from cm_read_results, with the reference's warnings."""
    import warnings

    if coordination_number_only and not options.silent:
        warnings.warn("coordination_number_only was set to true, so the MDDF and KB integrals were not computed. "
                      "(to remove this warning use Options(silent=true))")
    if not coordination_number_only and res["zero_random_bins"] > 0 and not options.silent:
        warnings.warn("Ideal-gas histogram bins with zero samples. Increase n_random_samples, number of trajectory "
                      "frames, and/or bin size.")
    for k in ("d", "md_count", "md_count_random", "coordination_number", "coordination_number_random", "mddf", "kb",
              "rdf_count", "rdf_count_random", "sum_rdf_count", "sum_rdf_count_random", "rdf", "kb_rdf",
              "solute_group_count", "solute_group_count_random", "solvent_group_count", "solvent_group_count_random"):
        setattr(R, k, res[k])
    R.volume.total = res["volume_total"]
    R.volume.shell = res["volume_shell"]
    if not coordination_number_only:
        R.volume.bulk = res["volume_bulk"]
        R.volume.domain = res["volume_domain"]
        R.density.solvent_bulk = res["density_solvent_bulk"]
    R.density.solute = res["density_solute"]
    R.density.solvent = res["density_solvent"]
    return R


def _run_frames(eng: Engine, trajectory: Trajectory, to_compute, fw, batch_frames: int) -> None:
    if not to_compute:
        return
    if isinstance(trajectory, ArrayTrajectory):
        for b0 in range(0, len(to_compute), batch_frames):
            if os.path.isfile(STOP_FILE):
                break
            ids = to_compute[b0 : b0 + batch_frames]
            xs, xv, cells = trajectory.frame_arrays([i - 1 for i in ids])
            eng.submit(xs, None if eng.autocorrelation else xv, cells, weights=[fw[i - 1] for i in ids], frame_ids=ids)
        return
    if isinstance(trajectory, NamdDCD):
        _run_dcd_frames(eng, trajectory, to_compute, fw, batch_frames)
        return
    wanted = set(to_compute)
    last = max(to_compute)
    trajectory.opentraj()
    trajectory.firstframe()
    xs, xv, cells, ids = [], [], [], []

    def flush():
        if ids:
            eng.submit(np.stack(xs), None if eng.autocorrelation else np.stack(xv), np.stack(cells),
                       weights=[fw[i - 1] for i in ids], frame_ids=list(ids))
            xs.clear(); xv.clear(); cells.clear(); ids.clear()

    try:
        for iframe in range(1, last + 1):
            if os.path.isfile(STOP_FILE):
                break
            trajectory.nextframe()
            if iframe not in wanted:
                continue
            xs.append(np.array(trajectory.x_solute, dtype=np.float64))
            xv.append(np.array(trajectory.x_solvent, dtype=np.float64))
            cells.append(cell_matrix(trajectory.getunitcell()))
            ids.append(iframe)
            if len(ids) >= batch_frames:
                flush()
        flush()
    finally:
        trajectory.closetraj()


def _run_dcd_frames(eng: Engine, traj: NamdDCD, to_compute, fw, batch_frames: int) -> None:
    """DCD frames go to the engine as the bytes read from the file; the
    engine gathers the selections on the device (no host-side gather or
    float32 -> float64 conversion)."""
    lay = traj.dcd_layout()
    s = np.asarray(traj.solute.indices, dtype=np.int64) - 1
    v = None if eng.autocorrelation else np.asarray(traj.solvent.indices, dtype=np.int64) - 1
    eng.set_dcd_layout(solute_atoms=s, solvent_atoms=v, **lay)
    for b0 in range(0, len(to_compute), batch_frames):
        if os.path.isfile(STOP_FILE):
            break
        ids = to_compute[b0 : b0 + batch_frames]
        lo, hi = ids[0], ids[-1]
        if hi - lo + 1 == len(ids):           # consecutive frames: one read
            raw, cells = traj.read_raw(lo - 1, len(ids))
        else:                                 # strided frames: read each one
            parts = [traj.read_raw(i - 1, 1) for i in ids]
            raw = np.concatenate([p[0] for p in parts])
            cells = np.concatenate([p[1] for p in parts])
        eng.submit_dcd(raw, cells, weights=[fw[i - 1] for i in ids], frame_ids=ids)


def coordination_number(*args, **kw):
    """Coordination numbers (src/mddf.jl:539-585) when called with a trajectory;
    with a Result, the group coordination number of
    src/tools/coordination_number.jl:104-106."""
    from .contributions import coordination_number as cn_result

    if args and isinstance(args[0], Result):
        return cn_result(*args, **kw)
    if "coordination_number_only" in kw:
        raise ValueError(
            "The keyword argument `coordination_number_only` is not allowed in the `coordination_number` function. "
            "It is, by definition, set to `true` in this function."
        )
    return mddf(*args, coordination_number_only=True, **kw)
