"""Finalisation on the device (cm_read_results, finalize="device") against
the host restatement of finalresults! (src/results.jl:311-469) on the same
engine counts: every field to 1e-12 of its scale, for cross and self MDDFs,
both bulk definitions, custom groups, frame weights and coordination-number
runs, and the reference's warning for random bins without samples."""
import warnings

import numpy as np
import pytest

from helpers import golden

pytestmark = pytest.mark.gpu

FIELDS = ("d", "md_count", "md_count_random", "coordination_number", "coordination_number_random", "mddf", "kb",
          "rdf_count", "rdf_count_random", "sum_rdf_count", "sum_rdf_count_random", "rdf", "kb_rdf",
          "solute_group_count", "solute_group_count_random", "solvent_group_count", "solvent_group_count_random")


def close(a, b, rtol=1e-12):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape
    scale = np.max(np.abs(b)) if b.size else 0.0
    return np.all(np.abs(a - b) <= rtol * max(scale, 1e-300))


def both(cm, traj_fn, opts, **kw):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        Rh = cm.mddf(traj_fn(), opts, **kw)
        Rd = cm.mddf(traj_fn(), opts, finalize="device", **kw)
    for f in FIELDS:
        assert close(getattr(Rd, f), getattr(Rh, f)), f
    # every Result reports its run's guard band, re-evaluation rate and largest FP32 error
    for R in (Rh, Rd):
        st = R.engine_stats
        assert st["records_within_cutoff"] > 0 and 0.0 <= st["guard_rate"] < 1.0
        assert 0.0 <= st["max_fp32_error"] <= st["guard_band"]
    assert close(Rd.volume.shell, Rh.volume.shell)
    for got, want in ((Rd.volume.total, Rh.volume.total), (Rd.volume.bulk, Rh.volume.bulk),
                      (Rd.volume.domain, Rh.volume.domain), (Rd.density.solute, Rh.density.solute),
                      (Rd.density.solvent, Rh.density.solvent), (Rd.density.solvent_bulk, Rh.density.solvent_bulk)):
        assert close(got, want), (got, want)
    return Rh, Rd


def namd(cm):
    g = golden("namd_frames.npz")
    cells = np.array([np.diag([c[0], c[2], c[5]]) for c in g["cells"]])
    tmao = cm.AtomSelection.from_indices(list(range(1479, 4013)), natomspermol=14,
                                         group_names=[str(s) for s in g["tmao_names"]])
    water = cm.AtomSelection.from_indices(list(range(4013, 10013)), natomspermol=3)
    protein = cm.AtomSelection.from_indices(list(range(1, 1464)), nmols=1,
                                            group_atom_indices=[list(range(1 + 10 * k, min(1464, 11 + 10 * k)))
                                                                for k in range(147)])
    xw = np.repeat(g["water"].astype(np.float64)[None], 2, axis=0)
    return g, cells, tmao, water, protein, xw


@pytest.mark.parametrize("usecutoff", [False, True])
def test_cross_water_tmao(cm, gpu_ready, usecutoff):
    g, cells, tmao, water, _, xw = namd(cm)
    opts = cm.make_options(**(dict(cutoff=10.0, dbulk=8.0, usecutoff=True) if usecutoff else dict(dbulk=8.0)),
                           n_random_samples=20, seed=5, silent=True)
    both(cm, lambda: cm.ArrayTrajectory(tmao, water, solute_frames=g["tmao"].astype(np.float64), solvent_frames=xw,
                                        cells=cells), opts)


def test_self_tmao_with_frame_weights(cm, gpu_ready):
    g, cells, tmao, *_ = namd(cm)
    opts = cm.make_options(dbulk=9.0, n_random_samples=20, seed=5, silent=True)
    both(cm, lambda: cm.ArrayTrajectory(tmao, solute_frames=g["tmao"].astype(np.float64), cells=cells), opts,
         frame_weights=[0.7, 1.9])


def test_protein_custom_groups_atoms_layout(cm, gpu_ready):
    g, cells, tmao, _, protein, _ = namd(cm)
    opts = cm.make_options(dbulk=10.0, n_random_samples=30, seed=9, silent=True)
    both(cm, lambda: cm.ArrayTrajectory(protein, tmao, solute_frames=g["protein"].astype(np.float64),
                                        solvent_frames=g["tmao"].astype(np.float64), cells=cells), opts)


def test_coordination_number_only(cm, gpu_ready):
    g, cells, tmao, water, _, xw = namd(cm)
    opts = cm.make_options(dbulk=8.0, seed=5, silent=True)
    Rh, Rd = both(cm, lambda: cm.ArrayTrajectory(tmao, water, solute_frames=g["tmao"].astype(np.float64),
                                                 solvent_frames=xw, cells=cells), opts,
                  coordination_number_only=True)
    assert Rd.coordination_number[-1] > 0


def test_zero_random_bins_warn_as_on_the_host(cm, gpu_ready):
    g, cells, tmao, water, _, xw = namd(cm)
    opts = cm.make_options(dbulk=8.0, n_random_samples=1, seed=5, silent=False, lastframe=1)
    tr = cm.ArrayTrajectory(tmao, water, solute_frames=g["tmao"].astype(np.float64), solvent_frames=xw, cells=cells)
    with pytest.warns(UserWarning, match="zero samples"):
        cm.mddf(tr, opts, finalize="device")
