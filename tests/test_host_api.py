"""Host-side API against the reference's own unit tests: Options
(src/Options.jl:194-237), AtomSelection (src/AtomSelection.jl:374-433), shell
volume and radius (src/results.jl:259-281), convert_unitcell
(src/Trajectory.jl:83-102) and random_move! keeping internal distances in
orthorhombic and triclinic cells (src/rigid_body.jl:139-190), through the
oracle's eulermat and move (the placement arithmetic the engine reproduces
bit for bit)."""
import math

import numpy as np
import pytest


def test_options_defaults_and_bulk_range(cm):
    mk = cm.make_options
    o = mk()
    assert (o.dbulk, o.cutoff, o.usecutoff) == (10.0, 10.0, False)
    o = mk(bulk_range=(10.0, 14.0))
    assert (o.dbulk, o.cutoff, o.usecutoff) == (10.0, 14.0, True)
    o = mk(dbulk=10.0)
    assert (o.dbulk, o.cutoff, o.usecutoff) == (10.0, 10.0, False)
    o = mk(dbulk=10.0, usecutoff=False)
    assert (o.dbulk, o.cutoff, o.usecutoff) == (10.0, 10.0, False)
    assert mk(cutoff=12.0, usecutoff=True).cutoff == 12.0
    assert mk(dbulk=10.0, usecutoff=True).cutoff == 14.0


@pytest.mark.parametrize("kw", [
    dict(dbulk=10.0, binstep=0.3),
    dict(dbulk=10.0, cutoff=10.0, usecutoff=True),
    dict(dbulk=6.0, cutoff=10.0, binstep=0.3, usecutoff=True),
    dict(dbulk=8.0, cutoff=10.0, binstep=0.3, usecutoff=True),
    dict(bulk_range=(10.0, 12.0), binstep=0.3),
    dict(stride=0),
    dict(lastframe=1, firstframe=2),
    dict(bulk_range=(12.0, 10.0)),
    dict(bulk_range=(12.0, 10.0), dbulk=8.0),
    dict(bulk_range=(12.0, 10.0), cutoff=15.0),
    dict(bulk_range=(12.0, 10.0), usecutoff=False),
    dict(dbulk=10.0, cutoff=15.0, usecutoff=False),
    dict(n_random_samples=0),
    dict(bulk_range=[1.0]),
    dict(cutoff=12.0),
])
def test_options_input_errors(cm, kw):
    with pytest.raises(ValueError):
        cm.make_options(**kw)


def test_atomselection_indices(cm):
    s = cm.AtomSelection.from_indices([12 + i for i in range(1, 12)], nmols=1, natomspermol=11)
    assert s.indices == [12 + i for i in range(1, 12)]
    assert (s.natomspermol, s.nmols, s.custom_groups, s.group_names) == (11, 1, False, [])
    s = cm.AtomSelection.from_indices(list(range(13, 24)), group_names=["C"] * 11, nmols=1, natomspermol=11)
    assert s.custom_groups is False and s.group_names == ["C"] * 11
    with pytest.raises(ValueError):
        cm.atom_group(s, "C")
    # shuffled indices inside a custom group give the same group
    idx = list(range(1, 41))
    g = list(range(5, 15))
    s1 = cm.AtomSelection.from_indices(idx, nmols=1, group_atom_indices=[g])
    s2 = cm.AtomSelection.from_indices(idx, nmols=1, group_atom_indices=[list(reversed(g))])
    assert cm.atom_group(s1, 1) == cm.atom_group(s2, 1)


@pytest.mark.parametrize("args,kw", [
    (([1, 2, 3],), {}),
    (([1, 2, 3],), dict(natomspermol=2)),
    (([1, 2, 3],), dict(natomspermol=1, nmols=2)),
    (([1, 2, 3],), dict(natomspermol=1, group_names=["A", "B"])),
    (([1, 2, 3],), dict(natomspermol=1, group_names=["A", "B", "C"])),
    (([],), dict(nmols=1, natomspermol=11)),
    (([1, 2, 3],), dict(natomspermol=1, group_atom_indices=[[1, 2, 2], [3]])),
    (([1, 2, 3],), dict(nmols=1, group_names=["A", "B"], group_atom_indices=[[1], [2, 3], [2]])),
])
def test_atomselection_argument_errors(cm, args, kw):
    with pytest.raises(ValueError):
        cm.AtomSelection.from_indices(*args, **kw)


def test_shell_volume_and_radius(cm):
    v = cm.sphericalshellvolume
    assert math.isclose(v(1, 1.0), 4 * math.pi / 3)
    assert math.isclose(v(2, 1.0), 4 * math.pi / 3 * (8 - 1))
    assert math.isclose(v(3, 1.0), 4 * math.pi / 3 * (27 - 8))
    assert math.isclose(cm.shellradius(1, 0.1), 0.07937005259840998)
    assert math.isclose(cm.shellradius(5, 0.3), 1.3664650373440481)


def test_convert_unitcell(cm):
    assert np.asarray(cm.convert_unitcell(np.eye(3))).shape == (3,)
    m = np.array([[1.0, 1.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 2.0]])
    assert np.asarray(cm.convert_unitcell(m)).shape == (3, 3)


def _internal_distances(x):
    d = x[:, None, :] - x[None, :, :]
    return np.sqrt((d ** 2).sum(-1))


@pytest.mark.parametrize("H", [np.diag([10.0, 10.0, 10.0]),
                               np.array([[10.0, 5.0, 0.0], [0.0, 10.0, 0.0], [0.0, 0.0, 10.0]])],
                         ids=["orthorhombic", "triclinic"])
@pytest.mark.parametrize("shift", [-1.0, -9.0, 4.0])
def test_random_move_keeps_internal_distances(orc, H, shift):
    """A molecule made whole about its reference atom (minimum image in the
    cell), rotated by eulermat about its centre and moved to a random centre
    keeps its internal distances."""
    rng = np.random.default_rng(11)
    x = shift + 2.0 * rng.random((5, 3))
    for k in range(4):
        ref = x[0]
        d = x - ref
        f = np.linalg.solve(H, d.T).T          # minimum image about the reference atom
        whole = ref + d - (np.rint(f) @ H.T)
        ang = rng.uniform(0.0, 2 * np.pi, 3)
        A = orc.eulermat_cs(*(v for a in ang for v in (np.cos(a), np.sin(a))))
        centre = H @ rng.random(3)
        y = orc.move(whole, centre, A)
        assert np.allclose(_internal_distances(x), _internal_distances(y), rtol=1e-12, atol=1e-12)
        assert np.allclose(y.mean(axis=0), centre, atol=1e-12)


def test_frame_slices_keep_their_stride(cm):
    """A slice of a larger frame array is passed with its frame stride, a
    non-contiguous frame is copied (no GPU needed)."""
    eng = cm.engine
    big = np.zeros((3, 10, 3), dtype=np.float32)
    fr, keep = eng.frames_struct(big[:, :4], None, np.repeat(np.eye(3)[None], 3, 0), None, None, 4, 4, True)
    assert fr.solute_frame_stride == 30 and keep[0].base is not None
    fr, _ = eng.frames_struct(big[:, :4].copy(), None, np.repeat(np.eye(3)[None], 3, 0), None, None, 4, 4, True)
    assert fr.solute_frame_stride == 0
    fr, keep = eng.frames_struct(big[:, ::2], None, np.repeat(np.eye(3)[None], 3, 0), None, None, 5, 5, True)
    assert fr.solute_frame_stride == 0 and keep[0].flags["C_CONTIGUOUS"]
