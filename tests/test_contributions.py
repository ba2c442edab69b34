"""Group and residue contributions (src/tools/contributions.jl:70-248,
src/tools/residue_contributions.jl:157-373).

CPU: the resolution of SoluteGroup / SolventGroup into summed group rows, and
ResidueContributions on the host (residue runs, the dmin/dmax window, slicing,
iteration, arithmetic), restating the reference's own tests of those rules.
GPU: cm_contributions (one launch for many queries) against the host
restatement on the same run, to 1e-12 of each curve's scale, for all four
types, both sides, atom indices on single- and multi-molecule selections,
custom group names and self-MDDF, and ResidueContributions of a protein.
"""
import warnings

import numpy as np
import pytest

from helpers import golden


def _selections(cm, nres=8, apr=5):
    natoms = nres * apr
    protein = cm.AtomSelection.from_indices(list(range(1, natoms + 1)), nmols=1)
    water = cm.AtomSelection.from_indices(list(range(natoms + 1, natoms + 1 + 30)), natomspermol=3)
    return protein, water


def _result(cm, seed=3, nb=50):
    """A finalised-looking Result with random positive group counts."""
    protein, water = _selections(cm)
    rng = np.random.default_rng(seed)
    R = cm.Result(nbins=nb, dbulk=8.0, cutoff=10.0, autocorrelation=False, solute=protein, solvent=water, files=[],
                  weights=[1.0])
    R.d = (np.arange(nb) + 0.5) * 0.2
    R.solute_group_count = rng.random((protein.ngroups(), nb))
    R.solute_group_count_random = rng.random((protein.ngroups(), nb))
    R.solvent_group_count = rng.random((water.ngroups(), nb))
    R.solvent_group_count_random = rng.random((water.ngroups(), nb))
    R.md_count_random = rng.random(nb)
    R.md_count_random[[3, 7]] = 0.0
    R.density.solvent_bulk = 0.033
    return R


def _atoms(cm, nres=8, apr=5):
    n = nres * apr
    return cm.Atoms(np.zeros((n, 3)), name=[f"A{k % apr}" for k in range(n)], resname=["ALA"] * n,
                    chain=["A"] * n, resnum=[1 + k // apr for k in range(n)])


def test_terms_follow_the_reference_rules(cm):
    R = _result(cm)
    assert cm.contribution_terms(R, cm.SoluteGroup([4, 2])) == ("solute", [3, 1], False, 1)
    # without custom groups a group index or name is an error (src/tools/contributions.jl:117-133)
    with pytest.raises(ValueError, match="no custom group names"):
        cm.contribution_terms(R, cm.SoluteGroup(3))
    # custom groups: by index or name, one row
    custom = cm.AtomSelection.from_indices(list(range(1, 41)), nmols=1, group_atom_indices=[[1, 2], [3, 4, 5]],
                                           group_names=["head", "tail"])
    Rc = cm.Result(nbins=5, dbulk=8.0, cutoff=10.0, autocorrelation=False, solute=custom, solvent=R.solvent,
                   files=[], weights=[1.0])
    assert cm.contribution_terms(Rc, cm.SoluteGroup(2)) == ("solute", [1], False, 1)
    assert cm.contribution_terms(Rc, cm.SoluteGroup("head")) == ("solute", [0], False, 1)
    with pytest.raises(ValueError, match="Custom groups are defined"):
        cm.contribution_terms(Rc, cm.SoluteGroup([1, 2]))
    # water: 10 molecules of 3 atoms; atom indices count by atom type and divide by nmols
    side, rows, divide, nmols = cm.contribution_terms(R, cm.SolventGroup([41, 45]))
    assert (side, rows, divide, nmols) == ("solvent", [0, 1], True, 10)
    with pytest.raises(ValueError, match="repeated"):
        cm.contribution_terms(R, cm.SoluteGroup([1, 1]))
    with pytest.raises(ValueError, match="not found"):
        cm.contribution_terms(R, cm.SoluteGroup([400]))
    with pytest.raises(ValueError, match="greater than number of groups"):
        cm.contribution_terms(Rc, cm.SoluteGroup(3))


def test_host_sum_matches_explicit_loops(cm):
    R = _result(cm)
    atoms = [41, 43, 45]
    got = cm.contributions(R, cm.SolventGroup(atoms), type="md_count")
    want = np.zeros(R.nbins)
    for iat in atoms:
        want += R.solvent_group_count[(iat - 41) % 3] / 10
    np.testing.assert_array_equal(got, want)
    kbi = cm.contributions(R, cm.SoluteGroup([1, 2]), type="kbi")
    s = R.solute_group_count[0] + R.solute_group_count[1]
    sr = R.solute_group_count_random[0] + R.solute_group_count_random[1]
    want = cm.units.Angs3tocm3permol * (1 / 0.033) * (np.cumsum(s) - np.cumsum(sr))
    np.testing.assert_allclose(kbi, want, rtol=1e-14)
    mddf = cm.contributions(R, cm.SoluteGroup([1]))
    assert mddf[3] == 0.0 and mddf[7] == 0.0


def test_residue_contributions_host(cm):
    R = _result(cm)
    atoms = _atoms(cm)
    rc = cm.ResidueContributions(R, atoms, silent=True)
    # the window: from the first d > dmin to the first d > dmax, inclusive
    i0 = int(np.nonzero(R.d > 1.5)[0][0])
    i1 = int(np.nonzero(R.d > 3.5)[0][0])
    np.testing.assert_array_equal(rc.d, R.d[i0:i1 + 1])
    assert rc.resnums == list(range(1, 9)) and len(rc) == 8
    assert rc.xticks == (list(range(1, 9)), [f"ALA{k}" for k in range(1, 9)])
    full = cm.ResidueContributions(R, atoms, dmin=0.0, dmax=100.0, silent=True)
    assert len(full.d) == R.nbins
    for k in (0, 7):
        want = cm.contributions(R, cm.SoluteGroup(list(range(1 + 5 * k, 6 + 5 * k))))
        np.testing.assert_array_equal(full.residue_contributions[k], want)
    # indexing: a residue, a range, iteration over a single residue's distances
    r0 = rc[0]
    assert r0.resnums == [1] and len(r0) == len(rc.d)
    assert r0 == cm.ResidueContributions(R, atoms.take(np.array(atoms.resnum) == 1), silent=True)
    r2 = rc[1:4]
    assert r2.resnums == [2, 3, 4]
    assert r2 == cm.ResidueContributions(R, atoms.take([k for k in range(40) if 2 <= atoms.resnum[k] <= 4]),
                                         silent=True)
    assert list(r0) == list(rc.residue_contributions[0])
    assert sum(1 for _ in rc) == 8
    # arithmetic
    assert rc + rc == 2 * rc
    assert all(np.all(c == 0) for c in (rc - rc).residue_contributions)
    assert all(np.allclose(a, b, rtol=1e-15) for a, b in zip(((rc * 3) / 3).residue_contributions,
                                                             rc.residue_contributions))
    with pytest.warns(UserWarning, match="Division by zero"):
        q = rc / (rc - rc)
    assert all(np.all(c == 0) for c in q.residue_contributions)
    with pytest.raises(ValueError, match="empty"):
        cm.ResidueContributions(R, atoms.take(np.zeros(40, dtype=bool)), silent=True)


def close(a, b, rtol=1e-12):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b)) if b.size else 0.0
    return a.shape == b.shape and np.all(np.abs(a - b) <= rtol * max(scale, 1e-300))


def _namd(cm):
    g = golden("namd_frames.npz")
    cells = np.array([np.diag([c[0], c[2], c[5]]) for c in g["cells"]])
    return g, cells


@pytest.mark.gpu
@pytest.mark.parametrize("type", ["mddf", "coordination_number", "md_count", "kbi"])
def test_device_contributions_cross(cm, gpu_ready, type):
    g, cells = _namd(cm)
    # protein with custom groups (147 residue-like groups of 10 atoms); TMAO with per-atom groups named by atom
    protein = cm.AtomSelection.from_indices(list(range(1, 1464)), nmols=1,
                                            group_atom_indices=[list(range(1 + 10 * k, min(1464, 11 + 10 * k)))
                                                                for k in range(147)],
                                            group_names=[f"G{k + 1}" for k in range(147)])
    tmao = cm.AtomSelection.from_indices(list(range(1479, 4013)), natomspermol=14,
                                         group_names=[str(s) for s in g["tmao_names"]])
    opts = cm.make_options(dbulk=10.0, n_random_samples=10, seed=9, silent=True)
    tr = cm.ArrayTrajectory(protein, tmao, solute_frames=g["protein"].astype(np.float64),
                            solvent_frames=g["tmao"].astype(np.float64), cells=cells)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        R = cm.mddf(tr, opts, keep_engine=True)
    try:
        names = [str(x) for x in g["tmao_names"]]
        groups = [cm.SoluteGroup(5), cm.SoluteGroup("G12"), cm.SoluteGroup(147),
                  cm.SolventGroup(names[:2]), cm.SolventGroup(names[3:4]), cm.SolventGroup(list(range(1479, 1479 + 14 * 5, 2)))]
        hosts = [_host(cm, R, grp, type) for grp in groups]
        for grp, host in zip(groups, hosts):
            assert close(cm.contributions(R, grp, type=type), host), (grp, type)
        # all queries in one call, as the residue loop does
        q = [cm.contribution_terms(R, grp) for grp in groups]
        rows = R.engine.contributions([(s, type, r, d) for s, r, d, _ in q])
        for k, host in enumerate(hosts):
            assert close(rows[k], host), (k, type)
    finally:
        R.engine.close()


def _host(cm, R, grp, type):
    """The host restatement on the same Result (engine detached)."""
    eng, R.engine = R.engine, None
    try:
        return cm.contributions(R, grp, type=type)
    finally:
        R.engine = eng


@pytest.mark.gpu
def test_device_contributions_self_and_residues(cm, gpu_ready):
    g, cells = _namd(cm)
    tmao = cm.AtomSelection.from_indices(list(range(1479, 4013)), natomspermol=14,
                                         group_names=[str(s) for s in g["tmao_names"]])
    opts = cm.make_options(dbulk=9.0, n_random_samples=10, seed=5, silent=True)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        R = cm.mddf(cm.ArrayTrajectory(tmao, solute_frames=g["tmao"].astype(np.float64), cells=cells), opts,
                    finalize="device", keep_engine=True)
    eng = R.engine
    try:
        names = [str(x) for x in g["tmao_names"]]
        for grp in (cm.SoluteGroup(names[:3]), cm.SolventGroup(list(range(1479, 1479 + 28))), cm.SolventGroup([1490])):
            for type in ("mddf", "kbi"):
                assert close(cm.contributions(R, grp, type=type), _host(cm, R, grp, type)), (grp, type)
    finally:
        eng.close()
    # residues of the NAMD protein (10-atom residues), default per-atom groups
    protein = cm.AtomSelection.from_indices(list(range(1, 1464)), nmols=1)
    water = cm.AtomSelection.from_indices(list(range(4013, 10013)), natomspermol=3)
    xw = np.repeat(g["water"].astype(np.float64)[None], 2, axis=0)
    opts = cm.make_options(dbulk=8.0, n_random_samples=10, seed=7, silent=True)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        R = cm.mddf(cm.ArrayTrajectory(protein, water, solute_frames=g["protein"].astype(np.float64),
                                       solvent_frames=xw, cells=cells), opts, keep_engine=True)
    atoms = cm.Atoms(g["protein"][0].astype(np.float64), resname=["RES"] * 1463, chain=["A"] * 1463,
                     resnum=[1 + k // 10 for k in range(1463)])
    eng = R.engine
    try:
        # the reference's decomposition identities through the device path
        # (src/tools/contributions.jl:320-349): all solute atoms, the sum over
        # residues, a partition of the KBI, all solvent atoms, one molecule x nmols
        allp = list(range(1, 1464))
        assert close(cm.contributions(R, cm.SoluteGroup(allp)), R.mddf)
        rc_all = cm.ResidueContributions(R, atoms, dmin=0.0, dmax=100.0, silent=True)
        assert close(sum(rc_all.residue_contributions), R.mddf)
        kbi = cm.contributions(R, cm.SoluteGroup(allp[:700]), type="kbi") + cm.contributions(
            R, cm.SoluteGroup(allp[700:]), type="kbi")
        assert close(kbi, R.kb)
        assert close(cm.contributions(R, cm.SolventGroup(list(range(4013, 10013)))), R.mddf)
        assert close(R.solvent.nmols * cm.contributions(R, cm.SolventGroup([4013, 4014, 4015])), R.mddf)
        for type in ("mddf", "coordination_number"):
            dev = cm.ResidueContributions(R, atoms, dmin=0.0, dmax=10.0, type=type, silent=True)
            R.engine = None
            host = cm.ResidueContributions(R, atoms, dmin=0.0, dmax=10.0, type=type, silent=True)
            R.engine = eng
            assert len(dev) == 147 and dev.resnums == host.resnums
            for a, b in zip(dev.residue_contributions, host.residue_contributions):
                assert close(a, b)
    finally:
        eng.close()


def test_residue_contributions_save_load(cm, tmp_path):
    """save / load of ResidueContributions and the version rules of the
    reference's loader (src/tools/residue_contributions.jl:570-608)."""
    import json

    R = _result(cm)
    rc = cm.ResidueContributions(R, _atoms(cm), silent=True)
    f = tmp_path / "rc.json"
    assert "saved" in cm.save(str(f), rc)
    assert cm.load(str(f), cm.ResidueContributions) == rc
    cm.save(str(f), rc[0])
    one = cm.load(str(f), cm.ResidueContributions)
    assert one == rc[0] and len(one) == len(rc.d)
    f.write_text(json.dumps({"Version": "2.18.3"}))
    with pytest.raises(ValueError, match="does not appear"):
        cm.load(str(f), cm.ResidueContributions)
    for version in ("1000.0.0", "1.0.0"):
        D = rc.to_json()
        D["Version"] = version
        f.write_text(json.dumps(D))
        with pytest.raises(ValueError, match="version"):
            cm.load(str(f), cm.ResidueContributions)


def test_argument_errors_of_the_reference(cm):
    """The reference's contributions argument errors
    (src/tools/contributions.jl:269-314), on a custom-group solute and a
    per-atom solvent."""
    custom = cm.AtomSelection.from_indices(list(range(1, 41)), nmols=1,
                                           group_atom_indices=[[1, 2, 3], [4, 5], [6, 7, 8, 9], [10]],
                                           group_names=["acidic", "basic", "polar", "nonpolar"])
    water = cm.AtomSelection.from_indices(list(range(41, 71)), natomspermol=3, group_names=["OH2", "H1", "H2"])
    R = cm.Result(nbins=5, dbulk=8.0, cutoff=10.0, autocorrelation=False, solute=custom, solvent=water, files=[],
                  weights=[1.0])
    R.solute_group_count[:] = 1.0
    R.md_count_random[:] = 1.0
    assert np.all(cm.contributions(R, cm.SoluteGroup("acidic"), type="md_count") == 1.0)
    assert np.all(cm.contributions(R, cm.SoluteGroup(2), type="md_count") == 1.0)
    bad = [
        (cm.SolventGroup([41]), "wrong_type"),           # type must be one of the four
        (cm.SoluteGroup([1, 2, 3]), "mddf"),             # custom groups: no atom indices
        (cm.SoluteGroup(["N", "CA"]), "mddf"),           # custom groups: no atom names
        (cm.SolventGroup("acidic"), "mddf"),             # no custom solvent groups: no group name
        (cm.SolventGroup(1), "mddf"),                    # ... nor group index
        (cm.SolventGroup([5000]), "mddf"),               # atom index not in the selection
        (cm.SoluteGroup("NOT_FOUND"), "mddf"),           # group name not found
        (cm.SoluteGroup(1000), "mddf"),                  # group index beyond the groups
        (cm.SolventGroup([]), "mddf"),                   # empty selections
        (cm.SolventGroup(["NOT_FOUND"]), "mddf"),        # atom name not found
        (cm.SolventGroup([41, 41]), "mddf"),             # repeated indices
        (cm.SolventGroup(["OH2", "OH2"]), "mddf"),       # repeated names
    ]
    for grp, kind in bad:
        with pytest.raises(ValueError):
            cm.contributions(R, grp, type=kind)


def test_residue_window_lengths_of_the_reference(cm):
    """The reference's window sizes for binstep 0.02 and 500 bins
    (src/tools/residue_contributions.jl:549-561): 101 distances between the
    default dmin = 1.5 and dmax = 3.5, all 500 for dmin = 0 and dmax = 10."""
    R = _result(cm, nb=500)
    R.d = np.array([cm.shellradius(i, 0.02) for i in range(1, 501)])
    atoms = _atoms(cm)
    rc = cm.ResidueContributions(R, atoms, silent=True)
    assert len(rc.d) == 101 and all(len(c) == 101 for c in rc.residue_contributions)
    full = cm.ResidueContributions(R, atoms, dmin=0.0, dmax=10.0, silent=True)
    assert len(full.d) == 500 and full.d[0] == R.d[0] and full.d[-1] == R.d[-1]
    assert len(rc.xticks[0]) == len(rc.xticks[1]) == len(rc) == 8
