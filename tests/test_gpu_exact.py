"""Counts at the decision boundaries, GPU against the oracle, bin by bin.

The engine's counts are defined by the oracle's FP64 expression of a pair's
distance: the minimum over lattice images of |y - x - H n| on the input
coordinates, n searched around rint(H^-1 (y - x)) (CellListMap's contract
for pairwise!, restated at src/minimum_distances.jl:129-148), binned by
setbin (src/results.jl:28) and compared with the cutoff as d^2 <= cutoff^2.
These inputs put many pairs exactly on the boundaries where another rounding
of that distance would change a count:

* atoms on an integer lattice in cells with integer edge vectors, so every
  pair distance is the square root of an integer: the integer distances lie
  exactly on bin edges (d / 0.02 and d / 0.25 are whole numbers), pairs at
  exactly the cutoff (6) and at exactly dbulk (5) occur, and equal distances
  (argmin ties, src/minimum_distances.jl:30-39) are everywhere;
* the reference's cross.pdb toy system (solvent at exactly 9, 11 and 12
  Angstrom, src/mddf.jl:592-624), every histogram bin compared.

Both precisions, orthorhombic and triclinic cells, cross and self MDDFs and
both search layouts are covered; the random-insertion counts are compared as
well (their placements are not on the lattice).
"""
import numpy as np
import pytest

from helpers import KEYS, TRICLINIC, compare, golden, make_system

pytestmark = pytest.mark.gpu

ORTHO_INT = np.diag([24.0, 25.0, 26.0])
# columns a = (24, 0, 0), b = (12, 21, 0), c = (0, 0, 24): a triclinic cell with integer edge vectors
TRICLINIC_INT = np.array([[24.0, 12.0, 0.0], [0.0, 21.0, 0.0], [0.0, 0.0, 24.0]])

# rigid templates with integer atom offsets
T3 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=np.float64)
T5 = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [1, 1, 0], [1, 0, 1]], dtype=np.float64)


def signed_permutation(rng):
    P = np.eye(3)[rng.permutation(3)]
    return P * rng.choice([-1.0, 1.0], size=3)[:, None]


def lattice_mols(rng, n, template, box):
    """n copies of an integer template, rotated by signed axis permutations,
    anchored at integer points of [0, box)."""
    anchors = np.stack([rng.integers(0, int(b), size=n) for b in box], axis=1).astype(np.float64)
    out = np.empty((n, len(template), 3))
    for i in range(n):
        out[i] = anchors[i] + template @ signed_permutation(rng).T
    return out.reshape(-1, 3)


def lattice_chain(rng, n, start):
    """Self-avoiding walk of n atoms with unit steps along the axes."""
    steps = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], dtype=np.float64)
    pts = [np.asarray(start, dtype=np.float64)]
    seen = {tuple(pts[0])}
    while len(pts) < n:
        for k in rng.permutation(6):
            q = pts[-1] + steps[k]
            if tuple(q) not in seen:
                break
        pts.append(q)
        seen.add(tuple(q))
    return np.array(pts)


def lattice_frames(rng, x0, nframes, apm):
    """Frames of integer coordinates: the first as given, then whole-system
    integer shifts plus per-molecule shifts in {-1, 0, 1}."""
    out = [x0]
    nm = len(x0) // apm
    for _ in range(nframes - 1):
        shift = rng.integers(-3, 4, size=3).astype(np.float64)
        per = np.repeat(rng.integers(-1, 2, size=(nm, 3)), apm, axis=0).astype(np.float64)
        out.append(x0 + shift + per)
    return np.stack(out)


def box_of(H):
    return np.array([H[0, 0], H[1, 1], H[2, 2]])


OPT = dict(irefatom=2, cutoff=6.0, n_random_samples=6, seed=91)


def bins_for(binstep):
    return int(np.ceil(6.0 / binstep)) + 2


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("H", [ORTHO_INT, TRICLINIC_INT], ids=["ortho", "triclinic"])
@pytest.mark.parametrize("usecutoff", [False, True], ids=["dbulk=cutoff", "dbulk=5"])
@pytest.mark.parametrize("binstep", [0.02, 0.25])
def test_lattice_pairs_cross(cm, orc, gpu_ready, precision, H, usecutoff, binstep):
    rng = np.random.default_rng(101)
    xs0 = lattice_mols(rng, 12, T5, box_of(H))
    xv0 = lattice_mols(rng, 260, T3, box_of(H))
    xs = lattice_frames(rng, xs0, 2, 5)
    xv = lattice_frames(rng, xv0, 2, 3)
    cells = np.repeat(H[None], 2, axis=0)
    opt = dict(OPT, dbulk=5.0 if usecutoff else 6.0, usecutoff=usecutoff, binstep=binstep, nbins=bins_for(binstep))
    got, ref, _ = compare(cm, orc, ms=12, aps=5, mv=260, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False,
                          precision=precision, regime="pairs", groups="custom",
                          dtype=np.float32 if precision == "fp32" else np.float64, **opt)
    on_edge = ref["md"].reshape(-1)[np.arange(int(round(1 / binstep)) - 1, len(ref["md"]), int(round(1 / binstep)))]
    assert on_edge.sum() > 0 and ref["md_random"].sum() > 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("H", [ORTHO_INT, TRICLINIC_INT], ids=["ortho", "triclinic"])
def test_lattice_pairs_self(cm, orc, gpu_ready, precision, H):
    rng = np.random.default_rng(102)
    x0 = lattice_mols(rng, 150, T5, box_of(H))
    xs = lattice_frames(rng, x0, 2, 5)
    cells = np.repeat(H[None], 2, axis=0)
    opt = dict(OPT, dbulk=5.0, usecutoff=True, binstep=0.02, nbins=bins_for(0.02))
    got, ref, _ = compare(cm, orc, ms=150, aps=5, mv=150, apv=5, xs=xs, xv=None, cells=cells, self_mode=True,
                          precision=precision, regime="pairs", groups="custom", **opt)
    assert ref["md"].sum() > 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("H", [ORTHO_INT, TRICLINIC_INT], ids=["ortho", "triclinic"])
@pytest.mark.parametrize("sched", ["cell", "balanced"])
def test_lattice_atoms_cross(cm, orc, gpu_ready, precision, H, sched):
    rng = np.random.default_rng(103)
    chain = lattice_chain(rng, 60, box_of(H) // 2)
    xv0 = lattice_mols(rng, 300, T3, box_of(H))
    xs = lattice_frames(rng, chain, 2, 60)
    xv = lattice_frames(rng, xv0, 2, 3)
    cells = np.repeat(H[None], 2, axis=0)
    opt = dict(OPT, dbulk=5.0, usecutoff=True, binstep=0.02, nbins=bins_for(0.02))
    compare(cm, orc, ms=1, aps=60, mv=300, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False, precision=precision,
            regime="atoms", groups="custom", atoms_schedule=sched, **opt)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_lattice_atoms_self(cm, orc, gpu_ready, precision):
    rng = np.random.default_rng(104)
    x0 = np.concatenate([lattice_chain(rng, 40, rng.integers(0, 24, size=3)) for _ in range(10)])
    xs = lattice_frames(rng, x0, 2, 40)
    cells = np.repeat(TRICLINIC_INT[None], 2, axis=0)
    opt = dict(OPT, dbulk=6.0, usecutoff=False, binstep=0.25, nbins=bins_for(0.25))
    compare(cm, orc, ms=10, aps=40, mv=10, apv=40, xs=xs, xv=None, cells=cells, self_mode=True, precision=precision,
            regime="atoms", groups="custom", **opt)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("regime", ["pairs", "atoms"])
def test_toy_cross_every_bin(cm, orc, gpu_ready, precision, regime):
    """cross.pdb (src/mddf.jl:592-624): one atom at the origin, three waters
    whose atoms sit at exactly 9, 11 and 12 Angstrom along x in a 30 A box."""
    t = golden("toy.npz")
    xyz = t["cross_xyz"]
    xs = xyz[:, 9:10, :]
    xv = xyz[:, 0:9, :]
    cells = np.array([np.diag(c) for c in t["cross_cell"]])
    opt = dict(irefatom=1, cutoff=10.0, dbulk=10.0, usecutoff=False, binstep=0.02, nbins=500, n_random_samples=200,
               seed=321)
    # the solute molecule has one atom: the ATOMS layout is forced for the second case
    got, ref, _ = compare(cm, orc, ms=1, aps=1, mv=3, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False,
                          precision=precision, regime=regime, **opt)
    # 9 A: bin 450 (1-based) holds the closest water; its two other atoms lie farther
    assert ref["md"][449] == 2 * 2 and ref["md"].sum() == 2 * 2
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("lattice", [True, False], ids=["lattice", "random"])
@pytest.mark.parametrize("self_mode", [False, True], ids=["cross", "self"])
def test_guard_queue_overflow_finishes_on_the_gpu(cm, orc, gpu_ready, lattice, self_mode):
    """A guard and edge queue of one record per compute chunk: nearly every
    chunk overflows it, is redone on the device without queues, and the
    counts are still the oracle's."""
    rng = np.random.default_rng(105)
    if lattice:
        H = TRICLINIC_INT
        xs = lattice_frames(rng, lattice_mols(rng, 40 if self_mode else 12, T5, box_of(H)), 3, 5)
        xv = None if self_mode else lattice_frames(rng, lattice_mols(rng, 260, T3, box_of(H)), 3, 3)
        cells = np.repeat(H[None], 3, axis=0)
    else:
        xs, xv, cells = make_system(rng, TRICLINIC, 40 if self_mode else 12, 5, 260, 3, 3, self_mode)
    mv, apv = (40, 5) if self_mode else (260, 3)
    opt = dict(OPT, dbulk=5.0, usecutoff=True, binstep=0.02, nbins=bins_for(0.02))
    got, ref, st = compare(cm, orc, ms=40 if self_mode else 12, aps=5, mv=mv, apv=apv, xs=xs, xv=xv, cells=cells,
                           self_mode=self_mode, precision="fp32", regime="pairs", groups="custom",
                           engine_kw=dict(guard_queue_capacity=1), **opt)
    assert ref["md"].sum() > 0
