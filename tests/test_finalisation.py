"""Host finalisation (src/results.jl:311-469) against the reference's own saved
Results (test/data/{NAMD,Gromacs,PDB}/*.json, fields in tests/golden/).

A saved Result holds the finalised values.  The normalisation is undone to
get the raw counters the frame loop leaves (md_count x nmols x Q, random
counts / density_fix x nrandom x Q, volume x Q, with Q the sum of the frame
weights read).  The package's finalresults is then run on them, and every
derived field must match the saved one to 1e-12 relative.
"""
import glob
import os

import numpy as np
import pytest

from helpers import GOLDEN

FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "json_*.npz")))


def rebuild(cm, z):
    """A Result with the raw counters behind a saved Result."""
    nb = int(z["nbins"])
    auto = bool(z["autocorrelation"])

    def sel(prefix):
        n, apm = int(z[prefix + "_nmols"]), int(z[prefix + "_natomspermol"])
        first = int(z[prefix + "_first_index"])
        names = [str(x) for x in z[prefix + "_group_names"]]
        return cm.AtomSelection(n, apm, list(range(first, first + n * apm)), False, [], names)

    solute, solvent = sel("solute"), sel("solvent")
    opts = cm.Options(firstframe=int(z["firstframe"]), stride=int(z["stride"]), binstep=float(z["binstep"]),
                      dbulk=float(z["dbulk"]), cutoff=float(z["cutoff"]), usecutoff=bool(z["usecutoff"]),
                      n_random_samples=int(z["n_random_samples"]), silent=True)
    fw = [float(x) for x in z["frame_weights"]]
    files = [cm.TrajectoryFileOptions("saved.json", opts, 1, int(z["lastframe_read"]), 0, fw)]
    R = cm.Result(nbins=nb, dbulk=float(z["dbulk"]), cutoff=float(z["cutoff"]), autocorrelation=auto, solute=solute,
                  solvent=solvent, files=files, weights=[1.0])
    Q = sum(fw[k - 1] for k in range(opts.firstframe, int(z["lastframe_read"]) + 1, opts.stride))
    nmols = solute.nmols
    nrand = opts.n_random_samples
    fix = float(z["density_solvent_bulk"]) / float(z["density_solvent"])
    R.md_count = z["md_count"] * (nmols * Q)
    R.rdf_count = z["rdf_count"] * (nmols * Q)
    R.md_count_random = z["md_count_random"] / fix * (nrand * Q)
    R.rdf_count_random = z["rdf_count_random"] / fix * (nrand * Q)
    R.solute_group_count = np.asarray(z["solute_group_count"]).reshape(-1, nb) * (nmols * Q)
    R.solute_group_count_random = np.asarray(z["solute_group_count_random"]).reshape(-1, nb) / fix * (nrand * Q)
    if not auto:
        R.solvent_group_count = np.asarray(z["solvent_group_count"]).reshape(-1, nb) * (nmols * Q)
        R.solvent_group_count_random = np.asarray(z["solvent_group_count_random"]).reshape(-1, nb) / fix * (nrand * Q)
    R.volume.total = float(z["volume_total"]) * Q
    return R, opts


def close(a, b, rtol=1e-12):
    """Agreement to rtol relative to the field's scale (its largest
    magnitude): KB integrals are differences of cumulative sums, so elements
    near zero carry the rounding of the large terms they cancel."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b)) if b.size else 0.0
    return np.all(np.abs(a - b) <= rtol * max(scale, 1e-300))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[5:-4] for p in FIXTURES])
def test_finalresults_reproduces_saved_results(cm, path):
    z = np.load(path, allow_pickle=False)
    R, opts = rebuild(cm, z)
    R = cm.finalresults(R, opts, coordination_number_only=False)
    for field in ("mddf", "kb", "rdf", "kb_rdf", "coordination_number", "coordination_number_random", "md_count",
                  "md_count_random", "sum_rdf_count", "sum_rdf_count_random", "d"):
        assert close(getattr(R, field), z[field]), field
    assert close(R.volume.shell, z["volume_shell"])
    for got, want in ((R.volume.total, z["volume_total"]), (R.volume.bulk, z["volume_bulk"]),
                      (R.volume.domain, z["volume_domain"]), (R.density.solvent, z["density_solvent"]),
                      (R.density.solute, z["density_solute"]), (R.density.solvent_bulk, z["density_solvent_bulk"])):
        assert close(got, want), (got, float(want))


def test_fixtures_present():
    assert len(FIXTURES) == 6


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[5:-4] for p in FIXTURES])
def test_contributions_of_all_atoms_sum_to_the_mddf(cm, path):
    """Contribution identities the reference checks
    (src/tools/contributions.jl:320-349): the contributions of all solute
    atoms, and of all solvent atoms, add up to the MDDF, the coordination
    number and the md counts; one solvent molecule's atoms give 1/nmols."""
    z = np.load(path, allow_pickle=False)
    R, opts = rebuild(cm, z)
    R = cm.finalresults(R, opts, coordination_number_only=False)
    all_solute = cm.SoluteGroup(list(R.solute.indices))
    all_solvent = cm.SolventGroup(list(R.solvent.indices))
    for kind, ref in (("mddf", R.mddf), ("coordination_number", R.coordination_number), ("md_count", R.md_count)):
        for g in (all_solute, all_solvent):
            got = cm.contributions(R, g, type=kind)
            assert close(got, ref), (kind, type(g).__name__)
    # one molecule's atoms: 1/nmols of the total (the reference's per-residue identity)
    one = cm.SolventGroup(list(R.solvent.indices[: R.solvent.natomspermol]))
    assert close(R.solvent.nmols * cm.contributions(R, one), R.mddf)
    # the KB integral is the sum of the KBI contributions of a partition of the
    # solute atoms (src/tools/contributions.jl:327-330); atoms of one molecule
    # of a multi-molecule solute carry 1/nmols of it
    half = R.solute.natomspermol // 2 or 1
    mol = list(R.solute.indices[: R.solute.natomspermol])
    parts = [cm.contributions(R, cm.SoluteGroup(mol[:half]), type="kbi")]
    if mol[half:]:
        parts.append(cm.contributions(R, cm.SoluteGroup(mol[half:]), type="kbi"))
    assert close(R.solute.nmols * sum(parts), R.kb)
