"""save / load / merge of Results (src/results.jl:533-588, src/tools/merge.jl:10-150),
on the reference's own merge test (src/tools/merge.jl:152-190: the toy cross
system of two frames run as two Results and merged), computed through the
oracle; and save -> load round trips of finalised Results."""
import glob
import math
import os

import numpy as np
import pytest

from helpers import GOLDEN, golden, oracle_mddf


def _cross(cm):
    t = golden("toy.npz")
    x = t["cross_xyz"]
    cells = np.array([np.diag(c) for c in t["cross_cell"]])
    protein = cm.AtomSelection.from_indices([10], nmols=1)
    water = cm.AtomSelection.from_indices(list(range(1, 10)), natomspermol=3)
    return cm.ArrayTrajectory(protein, water, frames=x, cells=cells, filename="cross")


def approx(a, b):
    """Julia's default isapprox: relative tolerance sqrt(eps)."""
    return math.isclose(a, b, rel_tol=math.sqrt(np.finfo(float).eps))


def _fields_equal(A, B):
    for name in ("d", "md_count", "md_count_random", "coordination_number", "coordination_number_random", "mddf",
                 "kb", "solute_group_count", "solvent_group_count", "solute_group_count_random",
                 "solvent_group_count_random", "rdf_count", "rdf_count_random", "sum_rdf_count",
                 "sum_rdf_count_random", "rdf", "kb_rdf"):
        a, b = np.asarray(getattr(A, name)), np.asarray(getattr(B, name))
        assert a.shape == b.shape and np.array_equal(a, b, equal_nan=True), name
    assert A.density == B.density
    for k in ("total", "bulk", "domain"):
        assert getattr(A.volume, k) == getattr(B.volume, k)
    assert np.array_equal(A.volume.shell, B.volume.shell)
    assert (A.nbins, A.dbulk, A.cutoff, A.autocorrelation, A.weights) == (B.nbins, B.dbulk, B.cutoff, B.autocorrelation,
                                                                          B.weights)
    assert A.solute == B.solute and A.solvent == B.solvent
    assert A.files == B.files


def test_merge_of_two_frames_of_the_toy_system(cm, orc, tmp_path):
    """src/tools/merge.jl:152-190 with the oracle computing each part."""
    o1 = cm.make_options(seed=321, StableRNG=True, nthreads=1, silent=True, n_random_samples=10**5, lastframe=1)
    o2 = cm.make_options(seed=321, StableRNG=True, nthreads=1, silent=True, n_random_samples=10**5, firstframe=2)
    R1 = oracle_mddf(cm, orc, _cross(cm), o1)
    R2 = oracle_mddf(cm, orc, _cross(cm), o2)
    R = cm.merge([R1, R2])
    assert R.volume.total == 27000.0
    assert approx(R.volume.domain, R.volume.total - R.volume.bulk)
    assert math.isclose(R.volume.domain, (4 * math.pi / 3) * R.dbulk ** 3, rel_tol=0.01)
    assert approx(R.density.solute, 1 / R.volume.total)
    assert approx(R.density.solvent, 3 / R.volume.total)
    # the reference's two parts draw the same random placements (one frame
    # each, same seed), so their bulk volumes are equal and the averaged
    # bulk density is exactly 2 / bulk; the random stream here is keyed by
    # frame id, so the two bulk volumes differ by the Monte Carlo noise of
    # 10^5 samples and the average of the ratios only agrees to that order
    assert math.isclose(R.density.solvent_bulk, 2 / R.volume.bulk, rel_tol=1e-5)
    assert R.density.solvent_bulk == 0.5 * R1.density.solvent_bulk + 0.5 * R2.density.solvent_bulk
    assert R.weights == [0.5, 0.5]
    path = str(tmp_path / "merged.json")
    cm.save(path, R)
    _fields_equal(R, cm.load(path))
    # frame weights given for the frames: the file weights stay the frame shares
    R2w = oracle_mddf(cm, orc, _cross(cm), o2, frame_weights=[0.0, 2.0])
    with pytest.warns(UserWarning):
        Rw = cm.merge([R1, R2w])
    assert Rw.weights == [0.5, 0.5] and len(Rw.files) == 2


def test_merge_rejects_incompatible_results(cm, orc):
    o1 = cm.make_options(seed=321, silent=True, n_random_samples=10, lastframe=1)
    R1 = oracle_mddf(cm, orc, _cross(cm), o1)
    o2 = cm.make_options(seed=321, silent=True, n_random_samples=10, lastframe=1, binstep=0.05)
    R2 = oracle_mddf(cm, orc, _cross(cm), o2)
    with pytest.raises(ValueError):
        cm.merge([R1, R2])
    with pytest.raises(ValueError):
        cm.merge([])


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "json_*.npz"))),
                         ids=lambda p: os.path.basename(p)[5:-4])
def test_save_load_round_trip(cm, tmp_path, path):
    from test_finalisation import rebuild

    z = np.load(path, allow_pickle=False)
    R, opts = rebuild(cm, z)
    R = cm.finalresults(R, opts, coordination_number_only=False)
    out = str(tmp_path / "r.json")
    assert "saved" in cm.save(out, R)
    _fields_equal(R, cm.load(out))


def test_load_rejects_other_json(cm, tmp_path):
    p = tmp_path / "x.json"
    p.write_text('{"a": 1}')
    with pytest.raises(ValueError):
        cm.load(str(p))


def test_snapshot_from_saved_result_recovers_half_units(cm, orc, tmp_path):
    """A finalised Result, saved as JSON and loaded, gives back the exact
    half-unit counts behind it (the resume snapshot), here against the
    oracle's counts for the same frames."""
    from helpers import KEYS, TRICLINIC, make_system, system_kwargs

    rng = np.random.default_rng(33)
    xs, xv, cells = make_system(rng, TRICLINIC, 10, 4, 150, 3, 3, False)
    solute = cm.AtomSelection.from_indices(list(range(1, 41)), natomspermol=4)
    solvent = cm.AtomSelection.from_indices(list(range(41, 491)), natomspermol=3)
    traj = cm.ArrayTrajectory(solute, solvent, solute_frames=xs, solvent_frames=xv, cells=cells)
    opts = cm.make_options(seed=43, silent=True, n_random_samples=6, dbulk=6.0, binstep=0.02)
    R = oracle_mddf(cm, orc, traj, opts)
    path = str(tmp_path / "r.json")
    cm.save(path, R)
    snap = cm.snapshot_from_result(cm.load(path))
    tmeta = cm.trajectory_metadata(traj, opts)
    kw = system_kwargs(cm.new_result(traj, opts, tmeta, None), opts, tmeta.irefatom)
    ref = orc.run(ms=10, aps=4, mv=150, apv=3, solute_xyz=xs, solvent_xyz=xv, cells=cells, frame_ids=[1, 2, 3], **kw)
    for k in KEYS:
        assert np.array_equal(snap[k], ref[k]), k
    assert snap["frames"] == 3 and snap["frame_weight"] == 1.0
    assert math.isclose(snap["volume_total"], sum(orc.cell_volume(c) for c in cells), rel_tol=1e-14)
