"""The candidate grid of a single solute molecule (ATOMS layout, FP32 search)
against the CPU oracle, bin by bin.

Every grid subdivision, the grid switched off, frames whose lists overflow
the grid's capacity (they walk the stencil instead), orthorhombic and
triclinic cells, both bulk definitions, sparse and dense solutes, and integer
lattices whose distances sit exactly on bin edges, at the cutoff and in ties.
"""
import numpy as np
import pytest

from helpers import KEYS, ORTHO, TRICLINIC, compare, make_system
from test_gpu_exact import OPT, T3, TRICLINIC_INT, ORTHO_INT, bins_for, box_of, lattice_chain, lattice_frames, lattice_mols

pytestmark = pytest.mark.gpu

COMMON = dict(binstep=0.02, nbins=350, seed=91)


def chain_system(rng, H, n=400, nframes=2, mv=350, apv=3, confined=None, spread=0.9):
    steps = rng.normal(size=(n, 3))
    chain = np.cumsum(steps / np.linalg.norm(steps, axis=1, keepdims=True) * 1.53, axis=0)
    if confined is not None:
        # a compact solute: the walk folded into a sphere of radius `confined`
        r = np.linalg.norm(chain - chain.mean(axis=0), axis=1, keepdims=True)
        chain = (chain - chain.mean(axis=0)) * np.minimum(1.0, confined / np.maximum(r, 1e-9))
    chain = chain - chain.mean(axis=0) + H @ np.full(3, 0.5)
    xs = np.stack([chain + rng.normal(scale=0.2, size=chain.shape) for _ in range(nframes)])
    _, xv, cells = make_system(rng, H, 1, 1, mv, apv, nframes, False, spread=spread)
    return xs, xv, cells


@pytest.mark.parametrize("grid", [-1, 1, 2, 4, 6])
@pytest.mark.parametrize("H", [ORTHO, TRICLINIC], ids=["ortho", "triclinic"])
def test_grid_subdivisions_match_oracle(cm, orc, gpu_ready, grid, H):
    rng = np.random.default_rng(11)
    xs, xv, cells = chain_system(rng, H)
    opt = dict(irefatom=2, cutoff=6.0, dbulk=6.0, usecutoff=False, n_random_samples=6, **COMMON)
    got, ref, st = compare(cm, orc, ms=1, aps=400, mv=350, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False,
                           precision="fp32", regime="atoms", groups="custom", engine_kw=dict(atoms_grid=grid), **opt)
    assert ref["md"].sum() > 0 and ref["md_random"].sum() > 0 and ref["rdf_random"].sum() > 0


@pytest.mark.parametrize("capacity", [1, 5000])
def test_grid_overflow_walks_the_stencil(cm, orc, gpu_ready, capacity):
    """A list capacity below one frame's entries: those frames lose their grid
    and their molecule pairs take the walk path, with the oracle's counts."""
    rng = np.random.default_rng(12)
    xs, xv, cells = chain_system(rng, TRICLINIC, nframes=3)
    opt = dict(irefatom=1, cutoff=6.0, dbulk=4.5, usecutoff=True, n_random_samples=4, **COMMON)
    compare(cm, orc, ms=1, aps=400, mv=350, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False, precision="fp32",
            regime="atoms", groups="custom", engine_kw=dict(atoms_grid=3, atoms_grid_capacity=capacity), **opt)


@pytest.mark.parametrize("usecutoff", [False, True])
@pytest.mark.parametrize("dense", [False, True], ids=["sparse", "dense"])
def test_grid_bulk_rules_and_density(cm, orc, gpu_ready, usecutoff, dense):
    rng = np.random.default_rng(13)
    xs, xv, cells = chain_system(rng, ORTHO, n=600, mv=400, confined=6.0 if dense else None)
    opt = dict(irefatom=3, cutoff=6.5, dbulk=4.0 if usecutoff else 6.5, usecutoff=usecutoff, n_random_samples=5,
               **COMMON)
    got, ref, _ = compare(cm, orc, ms=1, aps=600, mv=400, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False,
                          precision="fp32", regime="atoms", dtype=np.float32, **opt)
    assert ref["md"].sum() > 0


def test_grid_four_site_solvent_and_default_groups(cm, orc, gpu_ready):
    """Solvent molecules of 5 atoms (more sites than one site group), default
    groups, five frames."""
    rng = np.random.default_rng(14)
    xs, xv, cells = chain_system(rng, TRICLINIC, n=250, nframes=5, mv=200, apv=5)
    opt = dict(irefatom=4, cutoff=5.5, dbulk=5.5, usecutoff=False, n_random_samples=3, **COMMON)
    compare(cm, orc, ms=1, aps=250, mv=200, apv=5, xs=xs, xv=xv, cells=cells, self_mode=False, precision="fp32",
            regime="atoms", **opt)


@pytest.mark.parametrize("H", [ORTHO_INT, TRICLINIC_INT], ids=["ortho", "triclinic"])
@pytest.mark.parametrize("grid", [2, 5])
def test_grid_lattice_edges_and_ties(cm, orc, gpu_ready, H, grid):
    """Integer lattices: every distance the square root of an integer, many on
    a bin edge, at the cutoff or tied; the grid decides only the records away
    from them and the rest go to the exact scan."""
    rng = np.random.default_rng(15)
    chain = lattice_chain(rng, 80, box_of(H) // 2)
    xv0 = lattice_mols(rng, 300, T3, box_of(H))
    xs = lattice_frames(rng, chain, 2, 80)
    xv = lattice_frames(rng, xv0, 2, 3)
    cells = np.repeat(H[None], 2, axis=0)
    opt = dict(OPT, dbulk=5.0, usecutoff=True, binstep=0.02, nbins=bins_for(0.02))
    got, ref, st = compare(cm, orc, ms=1, aps=80, mv=300, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False,
                           precision="fp32", regime="atoms", groups="custom", dtype=np.float32,
                           engine_kw=dict(atoms_grid=grid), **opt)
    assert st["guard_reevaluations"] > 0 and ref["md"].sum() > 0


def test_grid_and_walk_agree_with_stats(cm, orc, gpu_ready):
    """The grid path evaluates far fewer atom pairs than the walk for a chain
    in a large box, with identical counts."""
    rng = np.random.default_rng(16)
    H = np.diag([40.0, 40.0, 40.0])
    xs, xv, cells = chain_system(rng, H, n=500, mv=1500)
    opt = dict(irefatom=1, cutoff=8.0, dbulk=8.0, usecutoff=False, n_random_samples=4, **COMMON, )
    opt["nbins"] = 400
    g1, ref, s1 = compare(cm, orc, ms=1, aps=500, mv=1500, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False,
                          precision="fp32", regime="atoms", engine_kw=dict(atoms_grid=4), **opt)
    g2, _, s2 = compare(cm, orc, ms=1, aps=500, mv=1500, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False,
                        precision="fp32", regime="atoms", engine_kw=dict(atoms_grid=-1), **opt)
    for k in KEYS:
        assert np.array_equal(g1[k], g2[k]), k
    assert s1["atom_pairs_evaluated"] < s2["atom_pairs_evaluated"]


@pytest.mark.parametrize("apv,grid", [(3, 3), (3, -1), (14, 3)], ids=["water-grid", "water-walk", "large-grid"])
def test_random_insertion_placement_many_samples(cm, orc, gpu_ready, apv, grid):
    """Many random samples on fine bins: the random insertion's slots are
    placed in FP32 for small molecules (the band widened to match) and in FP64
    for large ones; the counts equal the oracle's bin by bin either way."""
    rng = np.random.default_rng(17)
    H = np.diag([32.0, 32.0, 32.0])
    mv = 1200 // apv
    # three-site molecules of water's size (centroid radius under 1 A), fourteen-site ones of about 3 A
    xs, xv, cells = chain_system(rng, H, n=300, nframes=2, mv=mv, apv=apv, spread=0.3 if apv == 3 else 0.9)
    opt = dict(irefatom=1, cutoff=7.0, dbulk=7.0, usecutoff=False, n_random_samples=24, binstep=0.01, nbins=700,
               seed=93)
    got, ref, st = compare(cm, orc, ms=1, aps=300, mv=mv, apv=apv, xs=xs, xv=xv, cells=cells, self_mode=False,
                           precision="fp32", regime="atoms", groups="custom", dtype=np.float32,
                           engine_kw=dict(atoms_grid=grid), **opt)
    assert ref["md_random"].sum() > 0 and st["guard_reevaluations"] > 0
