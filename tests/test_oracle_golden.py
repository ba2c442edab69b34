"""The CPU oracle pinned against the reference's own known answers.

Sources (paths in ComplexMixtures.jl):
  toy systems              src/mddf.jl:587-758
  coordination numbers     src/tools/coordination_number.jl:108-135 (frame 1 of
                           NAMD/trajectory.dcd, same as frame 1 of
                           NAMD/traj_duplicated_first_frame.dcd)
  default reference atom   src/results.jl:490, src/Trajectory.jl:262
  eulermat / move!         src/rigid_body.jl:59-65, 82-96
"""
import math
import os

import numpy as np
import pytest

from helpers import golden, oracle_mddf


def _toy(cm, name, nframes_pick=None):
    t = golden("toy.npz")
    x = t[name + "_xyz"]
    cells = np.array([np.diag(c) for c in t[name + "_cell"]])
    return x, cells


def _traj(cm, name, solute, solvent=None):
    x, cells = _toy(cm, name)
    return cm.ArrayTrajectory(solute, solvent, frames=x, cells=cells, filename=name)


@pytest.mark.parametrize("lastframe", [1, 2])
def test_toy_cross(cm, orc, lastframe):
    protein = cm.AtomSelection.from_indices([10], nmols=1)
    water = cm.AtomSelection.from_indices(list(range(1, 10)), natomspermol=3)
    opts = cm.make_options(seed=321, StableRNG=True, silent=True, n_random_samples=10**5, lastframe=lastframe)
    R = oracle_mddf(cm, orc, _traj(cm, "cross", protein, water), opts)
    assert R.volume.total == 27000.0
    assert math.isclose(R.volume.domain, R.volume.total - R.volume.bulk)
    assert math.isclose(R.volume.domain, (4 * math.pi / 3) * R.dbulk**3, rel_tol=0.01)
    assert math.isclose(R.density.solute, 1 / R.volume.total)
    assert math.isclose(R.density.solvent, 3 / R.volume.total)
    assert math.isclose(R.density.solvent_bulk, 2 / R.volume.bulk)
    assert math.isclose(R.md_count.sum(), 1)
    assert math.isclose(R.coordination_number.sum(), 51)
    C = oracle_mddf(cm, orc, _traj(cm, "cross", protein, water), opts, coordination_number_only=True)
    assert C.volume.total == R.volume.total
    assert C.volume.domain == 0.0
    assert math.isclose(C.density.solute, 1 / C.volume.total)
    assert math.isclose(C.density.solvent, 3 / C.volume.total)
    assert C.density.solvent_bulk == 0.0
    assert np.array_equal(C.md_count, R.md_count)
    assert np.array_equal(cm.coordination_number(C), cm.coordination_number(R))


def test_toy_frame_weights_errors(cm):
    protein = cm.AtomSelection.from_indices([10], nmols=1)
    water = cm.AtomSelection.from_indices(list(range(1, 10)), natomspermol=3)
    tr = _traj(cm, "cross", protein, water)
    tm = cm.trajectory_metadata(tr, cm.Options())
    with pytest.raises(ValueError):
        cm.new_result(tr, cm.Options(), tm, [1.0])
    atom = cm.AtomSelection.from_indices([1, 2], natomspermol=1)
    tr = _traj(cm, "self_monoatomic", atom)
    tm = cm.trajectory_metadata(tr, cm.Options())
    with pytest.raises(ValueError):
        cm.new_result(tr, cm.Options(), tm, [[0, 1], [0, 1]])
    for fw in ([0.0, 1.0], [False, True], [[0, 1]]):
        cm.new_result(tr, cm.Options(), tm, fw)


def test_toy_self(cm, orc):
    atom = cm.AtomSelection.from_indices([1, 2], natomspermol=1)
    opts = cm.make_options(seed=321, StableRNG=True, silent=True, n_random_samples=10**5, lastframe=1)
    R = oracle_mddf(cm, orc, _traj(cm, "self_monoatomic", atom), opts)
    assert R.volume.total == 27000.0
    assert math.isclose(R.volume.domain, R.volume.total - R.volume.bulk)
    assert math.isclose(R.volume.domain, (4 * math.pi / 3) * R.dbulk**3, rel_tol=0.1)
    assert math.isclose(R.density.solute, 2 / R.volume.total)
    assert math.isclose(R.density.solvent, 2 / R.volume.total)
    assert math.isclose(R.md_count.sum(), 1.0)
    R = oracle_mddf(cm, orc, _traj(cm, "self_monoatomic", atom), opts, coordination_number_only=True)
    assert math.isclose(R.md_count.sum(), 1.0)


def test_toy_self_bulk(cm, orc):
    atom = cm.AtomSelection.from_indices([1, 2], natomspermol=1)
    tr = lambda: _traj(cm, "self_monoatomic", atom)
    opts = cm.make_options(seed=321, StableRNG=True, silent=True, n_random_samples=10**5, firstframe=2)
    R = oracle_mddf(cm, orc, tr(), opts)
    assert R.volume.total == 27000.0
    assert math.isclose(R.volume.domain, (4 * math.pi / 3) * R.dbulk**3, rel_tol=0.1)
    assert math.isclose(R.density.solvent_bulk, 1 / R.volume.bulk)
    opts = cm.make_options(seed=321, StableRNG=True, silent=True, n_random_samples=10**5)
    R = oracle_mddf(cm, orc, tr(), opts)
    assert math.isclose(R.volume.domain, (4 * math.pi / 3) * R.dbulk**3, rel_tol=0.1)
    assert math.isclose(R.density.solute, 2 / R.volume.total)
    assert math.isclose(R.density.solvent_bulk, 0.5 / R.volume.bulk)


def test_toy_frame_weight_equivalences(cm, orc):
    atom = cm.AtomSelection.from_indices([1, 2], natomspermol=1)
    tr = lambda name="self_monoatomic": _traj(cm, name, atom)
    o2 = cm.make_options(seed=321, StableRNG=True, silent=True, firstframe=2)
    o = cm.make_options(seed=321, StableRNG=True, silent=True)
    R1 = oracle_mddf(cm, orc, tr(), o2)
    R2 = oracle_mddf(cm, orc, tr(), o, frame_weights=[0.0, 1.0])
    assert np.array_equal(R1.md_count, R2.md_count) and np.array_equal(R1.rdf_count, R2.rdf_count)
    R1 = oracle_mddf(cm, orc, tr(), o)
    R2 = oracle_mddf(cm, orc, tr(), o, frame_weights=[0.3, 0.3])
    assert np.array_equal(R1.md_count, R2.md_count) and np.array_equal(R1.rdf_count, R2.rdf_count)
    o13 = cm.make_options(seed=321, StableRNG=True, silent=True, firstframe=1, lastframe=3)
    R1 = oracle_mddf(cm, orc, tr("self_monoatomic_duplicated_first_frame"), o13)
    R2 = oracle_mddf(cm, orc, tr(), o, frame_weights=[2.0, 1.0])
    assert np.array_equal(R1.md_count, R2.md_count) and np.array_equal(R1.rdf_count, R2.rdf_count)
    assert math.isclose(R2.md_count.sum(), 2 / 3)
    R2 = oracle_mddf(cm, orc, tr(), o, frame_weights=[1.0, 2.0])
    assert math.isclose(R2.md_count.sum(), 1 / 3)


def test_toy_interrupt(cm, orc):
    atom = cm.AtomSelection.from_indices([1, 2], natomspermol=1)
    R = oracle_mddf(cm, orc, _traj(cm, "self_monoatomic", atom), cm.Options(silent=True), stop=True)
    assert R.md_count.sum() == 0.0


def _namd(cm):
    g = golden("namd_frames.npz")
    protein = cm.AtomSelection.from_indices(list(range(1, 1464)), nmols=1)
    tmao = cm.AtomSelection.from_indices(list(range(1479, 4013)), natomspermol=14,
                                         group_names=[str(s) for s in g["tmao_names"]])
    cells = np.array([np.diag([c[0], c[2], c[5]]) for c in g["cells"]])
    tr = cm.ArrayTrajectory(protein, tmao, solute_frames=g["protein"].astype(np.float64),
                            solvent_frames=g["tmao"].astype(np.float64), cells=cells, filename="namd")
    return tr, protein, tmao


def test_namd_default_irefatom(cm):
    tr, protein, tmao = _namd(cm)
    assert cm.trajectory_metadata(tr, cm.Options()).irefatom == 1


def test_namd_coordination_number(cm, orc):
    tr, protein, tmao = _namd(cm)
    opts = cm.make_options(lastframe=1, seed=321, StableRNG=True, silent=True, n_random_samples=200)
    R = oracle_mddf(cm, orc, tr, opts, coordination_number_only=True, backend="cells")
    assert np.isclose(R.solute_group_count.sum(), R.solvent_group_count.sum())
    assert R.coordination_number[np.argmax(R.d > 3)] == 7.0
    assert R.coordination_number[np.argmax(R.d > 5)] == 14.0
    assert cm.coordination_number(R, cm.SolventGroup(["O1"])).sum() == 1171.0


def test_backends_agree(cm, orc):
    """The cells backend reports the same pairs and distances as the
    all-pairs backend (orthorhombic and triclinic, cross and self, groups)."""
    rng = np.random.default_rng(3)
    for H in (np.diag([21.0, 23.0, 22.0]), np.array([[22.0, 11.0, 0.0], [0.0, 19.05, 0.0], [0.0, 0.0, 22.0]])):
        for auto in (False, True):
            ms, aps, mv, apv = (30, 4, 30, 4) if auto else (3, 9, 40, 3)
            xs = (rng.random((2, ms, 1, 3)) @ H.T + rng.normal(scale=0.8, size=(2, ms, aps, 3))).reshape(2, -1, 3)
            xv = None if auto else (rng.random((2, mv, 1, 3)) @ H.T + rng.normal(scale=0.8, size=(2, mv, apv, 3))).reshape(2, -1, 3)
            cells = np.repeat(H[None], 2, axis=0)
            # custom groups: atom j of the selection is in groups j % 2 and 2; in
            # self mode the solvent table describes the same selection
            sg = [[a % 2, 2] for a in range(aps)]
            vg = [[j % 2, 2] for j in range(mv * apv)] if auto else None
            kw = dict(ms=ms, aps=aps, mv=mv, apv=apv, autocorrelation=auto, irefatom=2, cutoff=6.0, binstep=0.02,
                      dbulk=4.0, usecutoff=True, nbins=300, n_random_samples=3, seed=9, solute_xyz=xs, solvent_xyz=xv,
                      cells=cells, frame_ids=[4, 5], solute_groups=sg, solute_ngroups=3, solvent_groups=vg,
                      solvent_ngroups=3 if auto else 0)
            a = orc.run(backend="brute", **kw)
            b = orc.run(backend="cells", **kw)
            for k in ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
                      "solvent_group_random"):
                assert np.array_equal(a[k], b[k]), k
            assert a["md"].sum() > 0 and a["md_random"].sum() > 0


def test_eulermat_known(orc):
    """src/rigid_body.jl:59-65 with (cos, sin) of 0 and pi."""
    I = orc.eulermat_cs(1, 0, 1, 0, 1, 0)
    assert np.allclose(I, np.eye(3))
    assert np.allclose(orc.eulermat_cs(-1, 0, 1, 0, 1, 0), [[1, 0, 0], [0, -1, 0], [0, 0, -1]])
    assert np.allclose(orc.eulermat_cs(1, 0, -1, 0, 1, 0), [[-1, 0, 0], [0, 1, 0], [0, 0, -1]])
    assert np.allclose(orc.eulermat_cs(1, 0, 1, 0, -1, 0), [[-1, 0, 0], [0, -1, 0], [0, 0, 1]])


def test_move_known(orc):
    """src/rigid_body.jl:82-96."""
    x = np.array([[1.0, 0, 0], [0, 0, 0]])
    I = orc.eulermat_cs(1, 0, 1, 0, 1, 0)
    assert np.allclose(orc.move(x, [0, 0, 0], I), [[0.5, 0, 0], [-0.5, 0, 0]])
    assert np.allclose(orc.move(x, [1, 1, 1], I), [[1.5, 1, 1], [0.5, 1, 1]])
    assert np.allclose(orc.move(x, [0, 0, 0], orc.eulermat_cs(-1, 0, 1, 0, 1, 0)), [[0.5, 0, 0], [-0.5, 0, 0]])
    assert np.allclose(orc.move(x, [0, 0, 0], orc.eulermat_cs(1, 0, -1, 0, 1, 0)), [[-0.5, 0, 0], [0.5, 0, 0]])
    assert np.allclose(orc.move(x, [0, 0, 0], orc.eulermat_cs(1, 0, 1, 0, -1, 0)), [[-0.5, 0, 0], [0.5, 0, 0]])


def test_stream_spec(orc):
    """The documented stream: key() and SplitMix64 next(), restated in Python."""
    M = (1 << 64) - 1
    G = 0x9E3779B97F4A7C15

    def mix(z):
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    seed, tag, a, b, c = 321, 2, 7, 3, (1 << 32) | 5
    k = mix((seed + G * (tag + 1)) & M)
    for v in (a, b, c):
        k = mix(k ^ v)
    want = []
    for _ in range(6):
        k = (k + G) & M
        want.append(mix(k))
    assert list(orc.stream_draws(seed, tag, a, b, c, 6)) == want


def test_oracle_rejects_inconsistent_groups(orc):
    x = np.zeros((1, 4, 3))
    x[0, 2:, 0] = 3.0
    kw = dict(ms=2, aps=2, mv=2, apv=2, autocorrelation=True, irefatom=1, cutoff=5.0, binstep=0.02, dbulk=5.0,
              usecutoff=False, nbins=250, n_random_samples=1, seed=1, solute_xyz=x, solvent_xyz=None,
              cells=np.diag([20.0, 20.0, 20.0])[None], frame_ids=[1])
    with pytest.raises(ValueError):
        orc.run(solute_groups=[[0], [2]], solute_ngroups=3, **kw)
    with pytest.raises(ValueError):
        orc.run(solute_groups=[[0], [5]], solute_ngroups=3, solvent_groups=[[0]] * 4, solvent_ngroups=3, **kw)


def test_setbin_and_mindist(orc):
    assert orc.setbin(0.0, 0.02) == 1
    assert orc.setbin(9.0, 0.02) == 450
    assert orc.setbin(0.021, 0.02) == 2
    H = np.array([[10.0, 5.0, 0.0], [0.0, 8.660254037844386, 0.0], [0.0, 0.0, 10.0]])
    x = np.array([0.1, 0.2, 0.3])
    y = x + H @ np.array([1, -2, 1]) + np.array([0.5, -0.25, 0.0])
    assert math.isclose(orc.mindist2(H, x, y), 0.5**2 + 0.25**2, rel_tol=1e-12)
