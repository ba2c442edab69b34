"""Result and its FP64 finalisation (src/results.jl:10-118, 230-469, 629-649;
units from src/io.jl:6-14).  Host-side, O(nbins), unchanged semantics."""
from __future__ import annotations

import json
import math
import warnings
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .options import Options, TrajectoryFileOptions
from .selection import AtomSelection


class Units:
    """src/io.jl:6-14 (FP64 constants, derived the same way)."""

    mole = 6.022140857e23
    Angs3tocm3 = 1e24
    Angs3toL = 1e27
    Angs3tocm3permol = mole / Angs3tocm3
    Angs3toLpermol = mole / Angs3toL
    SitesperAngs3tomolperL = Angs3toL / mole


units = Units()


def setbin(d: float, step: float) -> int:
    """1-based histogram bin: max(1, ceil(d / step)) (src/results.jl:28)."""
    return max(1, int(math.ceil(d / step)))


def sphericalshellvolume(i: int, step: float) -> float:
    """Volume of the shell [(i-1) step, i step] (src/results.jl:254-257)."""
    rmin = (i - 1) * step
    return (4 * math.pi / 3) * ((rmin + step) ** 3 - rmin**3)


def shellradius(i: int, step: float) -> float:
    """Radius splitting the shell volume in halves (src/results.jl:272-275)."""
    rmin = (i - 1) * step
    return (0.5 * ((rmin + step) ** 3 + rmin**3)) ** (1 / 3)


@dataclass
class Density:
    solute: float = 0.0
    solvent: float = 0.0
    solvent_bulk: float = 0.0


@dataclass
class Volume:
    total: float
    bulk: float
    domain: float
    shell: np.ndarray


@dataclass
class Result:
    """Fields of src/results.jl:61-118.  Group counts are [ngroups, nbins]
    arrays (row g is group g+1 of the reference's Vector{Vector{Float64}})."""

    nbins: int
    dbulk: float
    cutoff: float
    autocorrelation: bool
    solute: AtomSelection
    solvent: AtomSelection
    files: List[TrajectoryFileOptions]
    weights: List[float]
    d: np.ndarray = None
    md_count: np.ndarray = None
    md_count_random: np.ndarray = None
    coordination_number: np.ndarray = None
    coordination_number_random: np.ndarray = None
    mddf: np.ndarray = None
    kb: np.ndarray = None
    solute_group_count: np.ndarray = None
    solvent_group_count: np.ndarray = None
    solute_group_count_random: np.ndarray = None
    solvent_group_count_random: np.ndarray = None
    rdf_count: np.ndarray = None
    rdf_count_random: np.ndarray = None
    sum_rdf_count: np.ndarray = None
    sum_rdf_count_random: np.ndarray = None
    rdf: np.ndarray = None
    kb_rdf: np.ndarray = None
    density: Density = field(default_factory=Density)
    volume: Volume = None
    Version: str = "2.18.3-DEV"

    def __post_init__(self):
        nb = self.nbins
        for name in (
            "d", "md_count", "md_count_random", "coordination_number", "coordination_number_random", "mddf", "kb",
            "rdf_count", "rdf_count_random", "sum_rdf_count", "sum_rdf_count_random", "rdf", "kb_rdf",
        ):
            if getattr(self, name) is None:
                setattr(self, name, np.zeros(nb))
        gs = self.solute.ngroups()
        gv = self.solvent.ngroups()
        if self.solute_group_count is None:
            self.solute_group_count = np.zeros((gs, nb))
        if self.solute_group_count_random is None:
            self.solute_group_count_random = np.zeros((gs, nb))
        if self.solvent_group_count is None:
            self.solvent_group_count = np.zeros((gv, nb))
        if self.solvent_group_count_random is None:
            self.solvent_group_count_random = np.zeros((gv, nb))
        if self.volume is None:
            self.volume = Volume(0.0, 0.0, 0.0, np.zeros(nb))


def isautocorrelation(solute_indices, solvent_indices) -> bool:
    """src/results.jl:240-243."""
    return list(solute_indices) == list(solvent_indices)


def check_frame_weights(frame_weights, options: Options, lastframe_read: int) -> np.ndarray:
    """Frame-weight validation of the Result constructor (src/results.jl:137-162)."""
    if frame_weights is None or len(np.asarray(frame_weights).reshape(-1)) == 0:
        return np.ones(lastframe_read)
    fw = np.asarray(frame_weights, dtype=np.float64)
    if sum(1 for s in fw.shape if s > 1) > 1:
        raise ValueError(
            f"The frame_weights provided must be one-dimensional, but a {fw.shape}-dimensional array was given."
        )
    fw = fw.reshape(-1)
    if len(fw) < lastframe_read:
        raise ValueError(
            "The length of the frame_weights vector provided must at least the number of frames to be read. "
            f"Input given: length(frame_weights) = {len(fw)}, last frame to be read: {lastframe_read}"
        )
    rng = range(options.firstframe, lastframe_read + 1, options.stride)
    if sum(fw[i - 1] for i in rng) <= 0.0:
        raise ValueError(
            "The sum of the frame weights must be greater than zero for the frames that will be considered."
        )
    return fw


def set_samples(R: Result):
    """src/results.jl:230-237."""
    nrand = R.files[0].options.n_random_samples
    if R.autocorrelation:
        return R.solvent.nmols - 1, nrand
    return R.solvent.nmols, nrand


def sum_frame_weights(R: Result) -> float:
    """src/results.jl:288-297."""
    Q = 0.0
    for f in R.files:
        i, s, l = f.options.firstframe, f.options.stride, f.lastframe_read
        Q += sum(f.frame_weights[k - 1] for k in range(i, l + 1, s))
    return Q


def finalresults(R: Result, options: Options, *, coordination_number_only: bool) -> Result:
    """src/results.jl:311-318.  Divisions follow IEEE semantics (x/0 gives
    Inf or NaN, as in the reference) instead of raising."""
    with np.errstate(divide="ignore", invalid="ignore"):
        if not coordination_number_only:
            return _mddf_final_results(R, options)
        return _coordination_number_final_results(R, options)


def _mddf_final_results(R: Result, options: Options) -> Result:
    """src/results.jl:320-376."""
    R.d = np.array([shellradius(i, options.binstep) for i in range(1, R.nbins + 1)])
    solvent_nmols, nrandom = set_samples(R)
    Q = sum_frame_weights(R)
    nmols = R.solute.nmols
    R.md_count = R.md_count / (nmols * Q)
    R.solute_group_count = R.solute_group_count / (nmols * Q)
    R.solute_group_count_random = R.solute_group_count_random / (nrandom * Q)
    if R.autocorrelation:
        R.solvent_group_count = R.solute_group_count.copy()
        R.solvent_group_count_random = R.solute_group_count_random.copy()
    else:
        R.solvent_group_count = R.solvent_group_count / (nmols * Q)
        R.solvent_group_count_random = R.solvent_group_count_random / (nrandom * Q)
    R.md_count_random = R.md_count_random / (nrandom * Q)
    R.rdf_count = R.rdf_count / (nmols * Q)
    R.rdf_count_random = R.rdf_count_random / (nrandom * Q)

    Q = np.float64(Q)
    R.volume.total = np.float64(R.volume.total) / Q
    R.volume.shell = R.volume.total * (R.rdf_count_random / solvent_nmols)
    binstep = R.files[0].options.binstep
    ibulk = setbin(R.dbulk + 0.5 * binstep, binstep)
    R.volume.domain = _jsum(R.volume.shell[: ibulk - 1])
    if not R.files[0].options.usecutoff:
        R.volume.bulk = R.volume.total - R.volume.domain
        n_solvent_in_bulk = solvent_nmols - _jsum(R.rdf_count)
    else:
        n_solvent_in_bulk = _jsum(R.rdf_count[ibulk - 1 : R.nbins])
        R.volume.bulk = _jsum(R.volume.shell[ibulk - 1 : R.nbins])
    R.density.solvent = float(R.solvent.nmols / np.float64(R.volume.total))
    R.density.solute = float(R.solute.nmols / np.float64(R.volume.total))
    R.density.solvent_bulk = float(np.float64(n_solvent_in_bulk) / np.float64(R.volume.bulk))
    density_fix = np.float64(R.density.solvent_bulk) / np.float64(R.density.solvent)
    R.volume.total = float(R.volume.total)
    return renormalize(R, density_fix, silent=options.silent)


def renormalize(R: Result, density_fix: float, *, silent: bool) -> Result:
    """src/results.jl:378-428."""
    R.md_count_random = R.md_count_random * density_fix
    R.rdf_count_random = R.rdf_count_random * density_fix
    R.solute_group_count_random = R.solute_group_count_random * density_fix
    R.solvent_group_count_random = R.solvent_group_count_random * density_fix
    R.coordination_number = _jcumsum(R.md_count)
    R.coordination_number_random = _jcumsum(R.md_count_random)
    warned = False
    nb = R.nbins
    mddf = np.zeros(nb) if R.mddf is None else R.mddf
    rdf = np.zeros(nb) if R.rdf is None else R.rdf
    kb = np.zeros(nb)
    kb_rdf = np.zeros(nb)
    srdf = np.zeros(nb)
    srdf_r = np.zeros(nb)
    f = units.Angs3tocm3permol
    inv = np.float64(1.0) / np.float64(R.density.solvent_bulk)
    for i in range(nb):
        if R.md_count_random[i] > 0.0:
            mddf[i] = R.md_count[i] / R.md_count_random[i]
        elif not warned and not silent:
            warnings.warn(
                "Ideal-gas histogram bins with zero samples. Increase n_random_samples, number of trajectory "
                "frames, and/or bin size."
            )
            warned = True
        kb[i] = f * inv * (R.coordination_number[i] - R.coordination_number_random[i])
        if R.rdf_count_random[i] > 0.0:
            rdf[i] = R.rdf_count[i] / R.rdf_count_random[i]
        if i == 0:
            srdf[i] = R.rdf_count[i]
            srdf_r[i] = R.rdf_count_random[i]
        else:
            srdf[i] = srdf[i - 1] + R.rdf_count[i]
            srdf_r[i] = srdf_r[i - 1] + R.rdf_count_random[i]
        kb_rdf[i] = f * inv * (srdf[i] - srdf_r[i])
    R.mddf, R.rdf, R.kb, R.kb_rdf, R.sum_rdf_count, R.sum_rdf_count_random = mddf, rdf, kb, kb_rdf, srdf, srdf_r
    return R


def _coordination_number_final_results(R: Result, options: Options) -> Result:
    """src/results.jl:430-469."""
    if not options.silent:
        warnings.warn(
            "coordination_number_only was set to true, so the MDDF and KB integrals were not computed. "
            "(to remove this warning use Options(silent=true))"
        )
    R.d = np.array([shellradius(i, options.binstep) for i in range(1, R.nbins + 1)])
    Q = sum_frame_weights(R)
    nmols = R.solute.nmols
    R.md_count = R.md_count / (nmols * Q)
    R.solute_group_count = R.solute_group_count / (nmols * Q)
    if R.autocorrelation:
        R.solvent_group_count = R.solute_group_count.copy()
    else:
        R.solvent_group_count = R.solvent_group_count / (nmols * Q)
    R.rdf_count = R.rdf_count / (nmols * Q)
    R.volume.total = float(np.float64(R.volume.total) / np.float64(Q))
    R.density.solvent = float(R.solvent.nmols / np.float64(R.volume.total))
    R.density.solute = float(R.solute.nmols / np.float64(R.volume.total))
    R.coordination_number = _jcumsum(R.md_count)
    R.sum_rdf_count = _jcumsum(R.rdf_count)
    return R


def sum_results(R1: Result, R2: Result) -> Result:
    """R1 += R2 for the raw counters (src/results.jl:629-649)."""
    R1.md_count += R2.md_count
    R1.md_count_random += R2.md_count_random
    R1.solute_group_count += R2.solute_group_count
    R1.solute_group_count_random += R2.solute_group_count_random
    R1.solvent_group_count += R2.solvent_group_count
    R1.solvent_group_count_random += R2.solvent_group_count_random
    R1.rdf_count += R2.rdf_count
    R1.rdf_count_random += R2.rdf_count_random
    R1.volume.total += R2.volume.total
    return R1


def _jsum(x) -> float:
    """Sum of a Float64 vector in index order.  Julia's Base.sum reduces
    pairwise above 1024 elements and lets LLVM reassociate below that, so
    results can differ from the reference in the last ulps; callers compare
    finalised fields at a relative tolerance of 1e-12."""
    s = 0.0
    for v in np.asarray(x, dtype=np.float64):
        s = s + float(v)
    return s


def _jcumsum(x) -> np.ndarray:
    out = np.empty(len(x))
    s = 0.0
    for i, v in enumerate(x):
        s = v if i == 0 else s + v
        out[i] = s
    return out


# ------------------------------------------------------------------ JSON
def result_from_json(path: str) -> Result:
    """Read a Result saved by the reference's ``save`` (JSON3 of the struct,
    src/results.jl:533-588).  Used to check the finalisation against saved
    results; the JSON fields map 1:1 onto the dataclass."""
    with open(path) as f:
        D = json.load(f)

    def sel(s):
        return AtomSelection(
            s["nmols"], s["natomspermol"], list(s["indices"]), bool(s["custom_groups"]),
            [list(g) for g in s["group_atom_indices"]], list(s["group_names"]),
        )

    files = []
    for ff in D["files"]:
        o = ff["options"]
        opts = Options(**{k: o[k] for k in Options.__dataclass_fields__ if k in o})
        files.append(
            TrajectoryFileOptions(ff["filename"], opts, ff["irefatom"], ff["lastframe_read"], ff["nframes_read"],
                                  list(ff["frame_weights"]))
        )
    R = Result(
        nbins=D["nbins"], dbulk=D["dbulk"], cutoff=D["cutoff"], autocorrelation=D["autocorrelation"],
        solute=sel(D["solute"]), solvent=sel(D["solvent"]), files=files, weights=list(D["weights"]),
        Version=D.get("Version", ""),
    )
    for k in ("d", "md_count", "md_count_random", "coordination_number", "coordination_number_random", "mddf", "kb",
              "rdf_count", "rdf_count_random", "sum_rdf_count", "sum_rdf_count_random", "rdf", "kb_rdf"):
        setattr(R, k, np.asarray(D[k], dtype=np.float64))
    for k in ("solute_group_count", "solvent_group_count", "solute_group_count_random", "solvent_group_count_random"):
        v = D[k]
        setattr(R, k, np.asarray(v, dtype=np.float64).reshape(len(v), -1) if len(v) else np.zeros((0, D["nbins"])))
    R.density = Density(**D["density"])
    v = D["volume"]
    R.volume = Volume(v["total"], v["bulk"], v["domain"], np.asarray(v["shell"], dtype=np.float64))
    return R


def _json_value(x):
    if isinstance(x, np.ndarray):
        return x.tolist()
    if isinstance(x, (np.floating, np.integer, np.bool_)):
        return x.item()
    return x


def result_to_json(R: Result) -> dict:
    """The fields of a Result in the reference's JSON layout and key order
    (JSON3 of the struct, src/results.jl:61-118, 533-540)."""
    def sel(a: AtomSelection):
        return {"nmols": a.nmols, "natomspermol": a.natomspermol, "indices": list(a.indices),
                "custom_groups": bool(a.custom_groups), "group_atom_indices": [list(g) for g in a.group_atom_indices],
                "group_names": list(a.group_names)}

    def rows(m):
        return [list(map(float, r)) for r in np.asarray(m, dtype=np.float64).reshape(-1, R.nbins)]

    files = []
    for f in R.files:
        o = f.options
        files.append({"filename": f.filename,
                      "options": {k: _json_value(getattr(o, k)) for k in Options.__dataclass_fields__},
                      "irefatom": f.irefatom, "lastframe_read": f.lastframe_read, "nframes_read": f.nframes_read,
                      "frame_weights": [float(w) for w in f.frame_weights]})
    v = R.volume
    return {
        "Version": R.Version, "nbins": R.nbins, "dbulk": float(R.dbulk), "cutoff": float(R.cutoff),
        "d": _json_value(R.d), "md_count": _json_value(R.md_count), "md_count_random": _json_value(R.md_count_random),
        "coordination_number": _json_value(R.coordination_number),
        "coordination_number_random": _json_value(R.coordination_number_random),
        "mddf": _json_value(R.mddf), "kb": _json_value(R.kb), "autocorrelation": bool(R.autocorrelation),
        "solute": sel(R.solute), "solvent": sel(R.solvent),
        "solute_group_count": rows(R.solute_group_count), "solvent_group_count": rows(R.solvent_group_count),
        "solute_group_count_random": rows(R.solute_group_count_random),
        "solvent_group_count_random": rows(R.solvent_group_count_random),
        "rdf_count": _json_value(R.rdf_count), "rdf_count_random": _json_value(R.rdf_count_random),
        "sum_rdf_count": _json_value(R.sum_rdf_count), "sum_rdf_count_random": _json_value(R.sum_rdf_count_random),
        "rdf": _json_value(R.rdf), "kb_rdf": _json_value(R.kb_rdf),
        "density": {"solute": float(R.density.solute), "solvent": float(R.density.solvent),
                    "solvent_bulk": float(R.density.solvent_bulk)},
        "volume": {"total": float(v.total), "bulk": float(v.bulk), "domain": float(v.domain),
                   "shell": _json_value(v.shell)},
        "files": files, "weights": [float(w) for w in R.weights],
    }


CURRENT_VERSION = (2, 18, 3)


def _version_tuple(v: str):
    """(major, minor, patch) of a version string such as "2.18.3" or "2.18.3-DEV"."""
    core = str(v).split("-")[0].split("+")[0]
    parts = [int(x) for x in core.split(".")[:3]]
    return tuple(parts + [0] * (3 - len(parts)))


def check_version(filename: str) -> None:
    """The reference's loading rules (src/io.jl:31-88): a file written by a
    newer version, or by one older than 2.0.0, is an argument error."""
    import os

    with open(os.path.expanduser(filename)) as f:
        try:
            v = json.load(f).get("Version", None)
        except (json.JSONDecodeError, AttributeError):
            return  # not JSON of a saved object: the loader reports it
    if v is None:
        return
    jv = _version_tuple(v)
    cur = ".".join(map(str, CURRENT_VERSION))
    if jv > CURRENT_VERSION:
        raise ValueError("Trying to load a json result file created with a newer version of ComplexMixtures. "
                         f"This can cause unpredictable errors. Current version of ComplexMixtures: {cur}. "
                         f"Version used to create the output .json file: {v}. Please update ComplexMixtures and try again.")
    if jv < (2, 0, 0):
        raise ValueError("Trying to load a json result created with an older, and incompatible, version of "
                         f"ComplexMixtures. Current version of ComplexMixtures: {cur}. Version used to create the "
                         f"output .json file: {v}.")


def save(filename: str, R) -> str:
    """Write a Result (or a ResidueContributions) as JSON that the reference's
    ``load`` reads (src/results.jl:533-540, src/tools/residue_contributions.jl:486-492);
    ``load`` here reads it back unchanged (floats are written with enough
    digits to round-trip)."""
    import os

    from .contributions import ResidueContributions

    filename = os.path.expanduser(filename)
    if isinstance(R, ResidueContributions):
        with open(filename, "w") as f:
            json.dump(R.to_json(), f, separators=(",", ":"), allow_nan=True)
        return f"ResidueContributions saved in JSON file: {filename}"
    with open(filename, "w") as f:
        json.dump(result_to_json(R), f, separators=(",", ":"), allow_nan=True)
    return f"Results saved in JSON file: {filename}"


def load(filename: str, kind=None):
    """Read a Result saved by ``save`` or by the reference (src/results.jl:567-588);
    ``load(filename, ResidueContributions)`` reads residue contributions
    (src/tools/residue_contributions.jl:509-528)."""
    import os

    check_version(filename)
    if kind is not None and kind is not Result:
        from .contributions import ResidueContributions

        if kind is not ResidueContributions:
            raise ValueError(f"load: unsupported type {kind}")
        try:
            with open(os.path.expanduser(filename)) as f:
                return ResidueContributions.from_json(json.load(f))
        except (KeyError, TypeError, ValueError, json.JSONDecodeError) as e:
            raise ValueError(f"The file {filename} does not appear to contain a ResidueContributions object.") from e
    try:
        return result_from_json(os.path.expanduser(filename))
    except (KeyError, TypeError, ValueError, json.JSONDecodeError) as e:
        raise ValueError(f"The file {filename} does not appear to contain a Result object.") from e


def snapshot_from_result(R: Result) -> dict:
    """The engine snapshot behind a finalised Result (``load`` of a saved
    JSON, src/results.jl:567-588): the normalisation of finalresults!
    (src/results.jl:320-376, 430-469) undone -- md/rdf/group counts times
    nmols x Q, random counts divided by density_fix and times nrandom x Q,
    volume times Q, with Q the sum of the frame weights -- and rounded to the
    exact half-unit integers of the frames' common weight.  ``Engine.restore``
    then resumes the run: frames submitted afterwards add to these counts.
    Results whose frames carry different weights cannot be resumed this way
    (``merge`` them instead)."""
    ws = [f.frame_weights[k - 1] for f in R.files
          for k in range(f.options.firstframe, f.lastframe_read + 1, f.options.stride) if f.frame_weights[k - 1] != 0.0]
    if not ws:
        raise ValueError("the Result holds no computed frame")
    w = float(ws[0])
    if any(float(x) != w for x in ws):
        raise ValueError("the Result's frames carry different weights: resume is defined for one frame weight "
                         "(merge the Results instead)")
    frames = len(ws)
    Q = sum_frame_weights(R)
    nmols = R.solute.nmols
    _, nrandom = set_samples(R)
    fix = np.float64(R.density.solvent_bulk) / np.float64(R.density.solvent) if R.density.solvent else 0.0

    def half_units(v, scale, random=False):
        v = np.asarray(v, dtype=np.float64)
        if random:
            if not np.any(v):
                return np.zeros(v.shape, dtype=np.int64)
            v = v / fix
        return np.rint(2.0 * (v * scale) / w).astype(np.int64)

    real, rand = nmols * Q, nrandom * Q
    snap = {
        "md": half_units(R.md_count, real), "md_random": half_units(R.md_count_random, rand, True),
        "rdf": half_units(R.rdf_count, real), "rdf_random": half_units(R.rdf_count_random, rand, True),
        "solute_group": half_units(R.solute_group_count, real),
        "solute_group_random": half_units(R.solute_group_count_random, rand, True),
    }
    if R.autocorrelation:
        snap["solvent_group"] = np.zeros_like(snap["solute_group"])
        snap["solvent_group_random"] = np.zeros_like(snap["solute_group_random"])
    else:
        snap["solvent_group"] = half_units(R.solvent_group_count, real)
        snap["solvent_group_random"] = half_units(R.solvent_group_count_random, rand, True)
    snap.update(frame_weight=w, frames=frames, volume_total=float(np.float64(R.volume.total) * np.float64(Q)))
    return snap


def merge(results: List[Result]) -> Result:
    """Average of Results of the same analysis over several trajectories or
    parts of one (src/tools/merge.jl:10-150): every function and counter is
    weighted by the frame weight of each Result over the total; ``weights``
    holds each file's share of the frames read."""
    if not results:
        raise ValueError("merge needs at least one Result")
    for i, a in enumerate(results):
        for b in results[i + 1:]:
            if a.nbins != b.nbins:
                raise ValueError("To merge Results, the number of bins of the histograms of the sets must be the same.")
            if not math.isclose(a.cutoff, b.cutoff, rel_tol=math.sqrt(np.finfo(float).eps)):
                raise ValueError("To merge Results, cutoff distance of the of the histograms of the sets must be the same.")
            if a.solute != b.solute or a.solvent != b.solvent:
                raise ValueError("To merge Results, the solute and solvent selections of the sets must be the same.")
            for name in ("solute_group_count", "solvent_group_count"):
                if np.shape(getattr(a, name)) != np.shape(getattr(b, name)):
                    raise ValueError(f"field {name} of the results are incompatible.")
    ntot_frames = sum(f.nframes_read for r in results for f in r.files)
    tot_frame_weight = sum(sum_frame_weights(r) for r in results)
    files = [f for r in results for f in r.files]
    weights = [f.nframes_read / ntot_frames for f in files]
    r0 = results[0]
    R = Result(nbins=r0.nbins, dbulk=r0.dbulk, cutoff=r0.cutoff, autocorrelation=r0.autocorrelation, solute=r0.solute,
               solvent=r0.solvent, files=files, weights=weights,
               solute_group_count=np.zeros_like(np.asarray(r0.solute_group_count, dtype=np.float64)),
               solvent_group_count=np.zeros_like(np.asarray(r0.solvent_group_count, dtype=np.float64)),
               solute_group_count_random=np.zeros_like(np.asarray(r0.solute_group_count, dtype=np.float64)),
               solvent_group_count_random=np.zeros_like(np.asarray(r0.solvent_group_count, dtype=np.float64)))
    R.d = np.array(r0.d, dtype=np.float64)
    warned = False
    for k, r in enumerate(results):
        w = sum_frame_weights(r) / tot_frame_weight
        if not math.isclose(w, R.weights[k], rel_tol=math.sqrt(np.finfo(float).eps)) and not warned:
            warned = True
            warnings.warn("Frame weights and file weights differ, because custom frame weights were provided.")
        for name in ("mddf", "kb", "rdf", "kb_rdf", "md_count", "md_count_random", "coordination_number",
                     "coordination_number_random", "solute_group_count", "solute_group_count_random",
                     "solvent_group_count", "solvent_group_count_random", "rdf_count", "rdf_count_random",
                     "sum_rdf_count", "sum_rdf_count_random"):
            setattr(R, name, getattr(R, name) + w * np.asarray(getattr(r, name), dtype=np.float64))
        R.density.solute += w * r.density.solute
        R.density.solvent += w * r.density.solvent
        R.density.solvent_bulk += w * r.density.solvent_bulk
        R.volume.total += w * r.volume.total
        R.volume.bulk += w * r.volume.bulk
        R.volume.domain += w * r.volume.domain
        R.volume.shell = R.volume.shell + w * np.asarray(r.volume.shell, dtype=np.float64)
    return R

