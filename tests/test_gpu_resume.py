"""Resume of a run from saved counts (src/results.jl:533-588 save / load,
src/tools/merge.jl:10-150 merge) through cm_load_raw_counts.

Frames 1..k on one engine, a snapshot written to a file, the snapshot
restored into a new engine and frames k+1..n added: the counts equal those of
one run over 1..n bit for bit (and the oracle's).  The same through a saved
JSON Result: its normalisation undone (snapshot_from_result), restored, the
rest of the frames added.  The merged Result of the two parts agrees with the
single run in every field that is linear in the counts.
"""
import numpy as np
import pytest

from helpers import KEYS, TRICLINIC, make_system

pytestmark = pytest.mark.gpu

SYS = dict(solute_nmols=40, solute_natomspermol=5, solvent_nmols=40, solvent_natomspermol=5, autocorrelation=True,
           irefatom=2, cutoff=7.0, binstep=0.02, dbulk=7.0, usecutoff=False, nbins=350, n_random_samples=4, seed=29)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_snapshot_restore_continue_equals_one_run(cm, orc, gpu_ready, tmp_path, precision):
    rng = np.random.default_rng(31)
    xs, _, cells = make_system(rng, TRICLINIC, 40, 5, 40, 5, 6, True)
    ids = list(range(1, 7))
    with cm.Engine(precision=precision, **SYS) as one:
        one.submit(xs, None, cells, frame_ids=ids)
        raw_all, counts_all = one.raw_counts(), one.counts()
    with cm.Engine(precision=precision, **SYS) as a:
        a.submit(xs[:3], None, cells[:3], frame_ids=ids[:3])
        path = cm.save_snapshot(str(tmp_path / "part1.npz"), a.snapshot())
    snap = cm.load_snapshot(path)
    assert snap["frames"] == 3 and snap["frame_weight"] == 1.0
    with cm.Engine(precision=precision, **SYS) as b:
        b.restore(snap)
        b.submit(xs[3:], None, cells[3:], frame_ids=ids[3:])
        raw_b, counts_b = b.raw_counts(), b.counts()
    for k in KEYS[:6]:
        assert np.array_equal(raw_b[k], raw_all[k]), k
    for k, v in counts_all.items():
        assert np.array_equal(np.asarray(counts_b[k]), np.asarray(v)), k
    opt = {k: SYS[k] for k in ("irefatom", "cutoff", "binstep", "dbulk", "usecutoff", "nbins", "n_random_samples", "seed")}
    ref = orc.run(ms=40, aps=5, mv=40, apv=5, solute_xyz=xs, solvent_xyz=None, cells=cells, frame_ids=ids,
                  autocorrelation=True, **opt)
    for k in KEYS[:6]:
        assert np.array_equal(raw_b[k], ref[k]), k


def test_resume_from_saved_json_result_and_merge(cm, gpu_ready, tmp_path):
    rng = np.random.default_rng(32)
    xs, xv, cells = make_system(rng, TRICLINIC, 12, 4, 200, 3, 6, False)
    solute = cm.AtomSelection.from_indices(list(range(1, 49)), natomspermol=4)
    solvent = cm.AtomSelection.from_indices(list(range(49, 649)), natomspermol=3)

    def traj():
        return cm.ArrayTrajectory(solute, solvent, solute_frames=xs, solvent_frames=xv, cells=cells)

    common = dict(seed=41, silent=True, n_random_samples=5, dbulk=6.0, binstep=0.02)
    R_all = cm.mddf(traj(), cm.make_options(**common), keep_engine=True)
    raw_all = R_all.engine.raw_counts()
    R_all.engine.close()
    R1 = cm.mddf(traj(), cm.make_options(lastframe=3, **common))
    cm.save(str(tmp_path / "part1.json"), R1)
    snap = cm.snapshot_from_result(cm.load(str(tmp_path / "part1.json")))
    assert snap["frames"] == 3
    o = cm.make_options(**common)
    tmeta = cm.trajectory_metadata(traj(), o)
    with cm.engine_for(R_all, o, tmeta.irefatom) as eng:
        eng.restore(snap)
        eng.submit(xs[3:], xv[3:], cells[3:], frame_ids=[4, 5, 6])
        raw = eng.raw_counts()
    for k in KEYS:
        assert np.array_equal(raw[k], raw_all[k]), k
    # merge of the two parts: the fields linear in the counts equal the one run's
    R2 = cm.mddf(traj(), cm.make_options(firstframe=4, **common))
    R = cm.merge([R1, R2])
    for f in ("md_count", "coordination_number", "rdf_count", "sum_rdf_count", "solute_group_count",
              "solvent_group_count"):
        a, b = np.asarray(getattr(R, f)), np.asarray(getattr(R_all, f))
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(b).max())), f
    assert np.isclose(R.volume.total, R_all.volume.total, rtol=1e-12)
