"""GPU engine (through the C ABI) against the CPU oracle, bit for bit.

Counts are int64 half units and must be identical.  Inputs are seeded random
molecular systems small enough for the oracle, covering orthorhombic and
triclinic cells, cross and self MDDFs, both search layouts, FP32+guard and
FP64, default and custom (overlapping) groups, and both bulk definitions.
"""
import numpy as np
import pytest

from helpers import KEYS, ORTHO, TRICLINIC, compare, golden, make_system, oracle_mddf

pytestmark = pytest.mark.gpu

COMMON = dict(binstep=0.02, nbins=350, seed=77)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("H", [ORTHO, TRICLINIC], ids=["ortho", "triclinic"])
@pytest.mark.parametrize("usecutoff", [False, True])
def test_pairs_self(cm, orc, gpu_ready, precision, H, usecutoff):
    rng = np.random.default_rng(1)
    xs, xv, cells = make_system(rng, H, 60, 5, 60, 5, 3, True)
    opt = dict(irefatom=2, cutoff=7.0, dbulk=5.0 if usecutoff else 7.0, usecutoff=usecutoff, n_random_samples=6,
               **COMMON)
    got, ref, st = compare(cm, orc, ms=60, aps=5, mv=60, apv=5, xs=xs, xv=None, cells=cells, self_mode=True,
                           precision=precision, regime="pairs", **opt)
    assert ref["md"].sum() > 0 and ref["md_random"].sum() > 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("H", [ORTHO, TRICLINIC], ids=["ortho", "triclinic"])
@pytest.mark.parametrize("groups", ["default", "custom"])
def test_pairs_cross(cm, orc, gpu_ready, precision, H, groups):
    rng = np.random.default_rng(2)
    xs, xv, cells = make_system(rng, H, 20, 7, 150, 3, 3, False)
    opt = dict(irefatom=1, cutoff=6.0, dbulk=6.0, usecutoff=False, n_random_samples=8, **COMMON)
    compare(cm, orc, ms=20, aps=7, mv=150, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False, precision=precision,
            regime="pairs", groups=groups, **opt)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("H", [ORTHO, TRICLINIC], ids=["ortho", "triclinic"])
@pytest.mark.parametrize("groups", ["default", "custom"])
def test_atoms_cross(cm, orc, gpu_ready, precision, H, groups):
    """A 300-atom solute molecule (ATOMS layout) in water-like solvent."""
    rng = np.random.default_rng(3)
    steps = rng.normal(size=(300, 3))
    chain = np.cumsum(steps / np.linalg.norm(steps, axis=1, keepdims=True) * 1.53, axis=0) + H @ np.full(3, 0.5)
    xs = np.stack([chain + rng.normal(scale=0.2, size=chain.shape) for _ in range(2)])
    _, xv, cells = make_system(rng, H, 1, 1, 300, 3, 2, False)
    opt = dict(irefatom=1, cutoff=6.0, dbulk=4.0, usecutoff=True, n_random_samples=5, **COMMON)
    compare(cm, orc, ms=1, aps=300, mv=300, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False, precision=precision,
            regime="atoms", groups=groups, **opt)


@pytest.mark.parametrize("regime", ["pairs", "atoms"])
def test_regimes_agree_self(cm, orc, gpu_ready, regime):
    """Self-MDDF through both layouts (the ATOMS layout handles it directionally)."""
    rng = np.random.default_rng(4)
    xs, _, cells = make_system(rng, TRICLINIC, 40, 6, 40, 6, 2, True)
    opt = dict(irefatom=3, cutoff=6.5, dbulk=6.5, usecutoff=False, n_random_samples=4, **COMMON)
    compare(cm, orc, ms=40, aps=6, mv=40, apv=6, xs=xs, xv=None, cells=cells, self_mode=True, precision="fp32",
            regime=regime, groups="custom", **opt)


def test_small_box_multi_image(cm, orc, gpu_ready):
    """Box narrower than twice the search range: several images per pair."""
    rng = np.random.default_rng(5)
    H = np.diag([13.0, 12.0, 14.0])
    xs, _, cells = make_system(rng, H, 12, 4, 12, 4, 2, True, spread=0.7)
    opt = dict(irefatom=1, cutoff=5.6, dbulk=5.6, usecutoff=False, n_random_samples=3, **COMMON)
    for regime in ("pairs", "atoms"):
        compare(cm, orc, ms=12, aps=4, mv=12, apv=4, xs=xs, xv=None, cells=cells, self_mode=True, precision="fp32",
                regime=regime, backend="brute", **opt)


def test_coordination_number_mode(cm, orc, gpu_ready):
    rng = np.random.default_rng(6)
    xs, xv, cells = make_system(rng, ORTHO, 10, 5, 120, 3, 2, False)
    opt = dict(irefatom=1, cutoff=6.0, dbulk=6.0, usecutoff=False, n_random_samples=3, coordination_number_only=True,
               **COMMON)
    got, ref, st = compare(cm, orc, ms=10, aps=5, mv=120, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False,
                           precision="fp32", regime="pairs", **opt)
    assert got["md_random"].sum() == 0 and ref["md"].sum() > 0


def test_fp32_coordinates(cm, orc, gpu_ready):
    """FP32-stored coordinates (the engine promotes them to FP64 exactly)."""
    rng = np.random.default_rng(7)
    xs, _, cells = make_system(rng, TRICLINIC * 2.0, 300, 14, 300, 14, 2, True, spread=1.5)
    opt = dict(irefatom=1, cutoff=8.0, dbulk=8.0, usecutoff=False, n_random_samples=5, **COMMON)
    compare(cm, orc, ms=300, aps=14, mv=300, apv=14, xs=xs, xv=None, cells=cells, self_mode=True, precision="fp32",
            regime="pairs", dtype=np.float32, **{**opt, "nbins": 400})


def test_fp32_equals_fp64_larger(cm, gpu_ready):
    """c3-like self system (2,000 molecules of 14 atoms, triclinic): the FP32 +
    guard path gives exactly the FP64 path's counts."""
    syn = cm_synth()
    s = syn.config3(nmols=2000, edge=64.4, nframes=3)
    xs, _, cells = s.frames()
    out = {}
    for prec in ("fp32", "fp64"):
        eng = __import__("complexmixtures_gb300").Engine(
            solute_nmols=2000, solute_natomspermol=14, solvent_nmols=2000, solvent_natomspermol=14,
            autocorrelation=True, irefatom=1, cutoff=10.0, binstep=0.02, dbulk=10.0, usecutoff=False, nbins=500,
            n_random_samples=5, seed=5, precision=prec)
        eng.submit(xs, None, cells)
        out[prec] = eng.raw_counts()
        st = eng.stats()
        eng.close()
    for k in KEYS[:6]:
        assert np.array_equal(out["fp32"][k], out["fp64"][k]), k
    assert out["fp32"]["md"].sum() > 0


def cm_synth():
    import importlib

    return importlib.import_module("complexmixtures_gb300.synth")


# ---------------------------------------------------------------- golden
def test_gpu_toy_cross(cm, gpu_ready):
    t = golden("toy.npz")
    protein = cm.AtomSelection.from_indices([10], nmols=1)
    water = cm.AtomSelection.from_indices(list(range(1, 10)), natomspermol=3)
    cells = np.array([np.diag(c) for c in t["cross_cell"]])
    for lastframe in (1, 2):
        tr = cm.ArrayTrajectory(protein, water, frames=t["cross_xyz"], cells=cells)
        opts = cm.make_options(seed=321, StableRNG=True, silent=True, n_random_samples=10**5, lastframe=lastframe)
        R = cm.mddf(tr, opts)
        assert R.volume.total == 27000.0
        assert np.isclose(R.volume.domain, (4 * np.pi / 3) * R.dbulk**3, rtol=0.01)
        assert np.isclose(R.density.solvent_bulk, 2 / R.volume.bulk)
        assert np.isclose(R.md_count.sum(), 1)
        assert np.isclose(R.coordination_number.sum(), 51)
        C = cm.coordination_number(cm.ArrayTrajectory(protein, water, frames=t["cross_xyz"], cells=cells), opts)
        assert np.array_equal(C.md_count, R.md_count)
        assert C.density.solvent_bulk == 0.0


def test_gpu_toy_self_and_weights(cm, orc, gpu_ready):
    t = golden("toy.npz")
    atom = cm.AtomSelection.from_indices([1, 2], natomspermol=1)
    tr = lambda n="self_monoatomic": cm.ArrayTrajectory(atom, frames=t[n + "_xyz"],
                                                        cells=np.array([np.diag(c) for c in t[n + "_cell"]]))
    o = cm.make_options(seed=321, StableRNG=True, silent=True)
    R = cm.mddf(tr(), cm.make_options(seed=321, silent=True, n_random_samples=10**5, lastframe=1))
    assert np.isclose(R.md_count.sum(), 1.0)
    assert np.isclose(R.volume.domain, (4 * np.pi / 3) * R.dbulk**3, rtol=0.1)
    R1 = cm.mddf(tr(), o)
    R2 = cm.mddf(tr(), o, frame_weights=[0.3, 0.3])
    assert np.array_equal(R1.md_count, R2.md_count) and np.array_equal(R1.rdf_count, R2.rdf_count)
    R1 = cm.mddf(tr("self_monoatomic_duplicated_first_frame"), cm.make_options(silent=True, lastframe=3))
    R2 = cm.mddf(tr(), o, frame_weights=[2.0, 1.0])
    assert np.array_equal(R1.md_count, R2.md_count)
    assert np.isclose(R2.md_count.sum(), 2 / 3)
    # finalised fields equal the oracle's through the same host code
    Ro = oracle_mddf(cm, orc, tr(), o, frame_weights=[2.0, 1.0])
    for f in ("md_count", "md_count_random", "rdf_count", "rdf_count_random", "mddf", "kb", "rdf", "kb_rdf"):
        assert np.array_equal(getattr(R2, f), getattr(Ro, f)), f


def test_gpu_namd_coordination_number(cm, gpu_ready):
    g = golden("namd_frames.npz")
    protein = cm.AtomSelection.from_indices(list(range(1, 1464)), nmols=1)
    tmao = cm.AtomSelection.from_indices(list(range(1479, 4013)), natomspermol=14,
                                         group_names=[str(s) for s in g["tmao_names"]])
    cells = np.array([np.diag([c[0], c[2], c[5]]) for c in g["cells"]])
    for precision in ("fp32", "fp64"):
        tr = cm.ArrayTrajectory(protein, tmao, solute_frames=g["protein"].astype(np.float64),
                                solvent_frames=g["tmao"].astype(np.float64), cells=cells)
        opts = cm.make_options(lastframe=1, seed=321, StableRNG=True, silent=True, n_random_samples=200)
        R = cm.mddf(tr, opts, precision=precision)
        assert np.isclose(R.solute_group_count.sum(), R.solvent_group_count.sum())
        assert R.coordination_number[np.argmax(R.d > 3)] == 7.0
        assert R.coordination_number[np.argmax(R.d > 5)] == 14.0
        assert cm.coordination_number(R, cm.SolventGroup(["O1"])).sum() == 1171.0


def test_gpu_namd_frames_vs_oracle(cm, orc, gpu_ready):
    """Real geometry: protein-TMAO (ATOMS layout) and TMAO-water (PAIRS) on two
    NAMD frames, MDDF with random insertion, bit for bit."""
    g = golden("namd_frames.npz")
    cells = np.array([np.diag([c[0], c[2], c[5]]) for c in g["cells"]])
    prot = g["protein"].astype(np.float64)
    tmao = g["tmao"].astype(np.float64)
    opt = dict(irefatom=1, cutoff=10.0, binstep=0.02, dbulk=8.0, usecutoff=True, nbins=500, n_random_samples=4,
               seed=321)
    compare(cm, orc, ms=1, aps=1463, mv=181, apv=14, xs=prot, xv=tmao, cells=cells, self_mode=False,
            precision="fp32", regime="atoms", **opt)
    water = np.repeat(g["water"].astype(np.float64)[None], 2, axis=0)
    compare(cm, orc, ms=181, aps=14, mv=2000, apv=3, xs=tmao, xv=water, cells=cells, self_mode=False,
            precision="fp32", regime="pairs", **opt)


@pytest.mark.parametrize("pct", [40, 60, 150])
@pytest.mark.parametrize("regime", ["pairs", "atoms"])
def test_cell_scale_does_not_change_counts(cm, orc, gpu_ready, pct, regime):
    """Search cells of another size (cell_scale_pct) give the same counts."""
    rng = np.random.default_rng(21)
    xs, xv, cells = make_system(rng, TRICLINIC, 30, 4, 200, 3, 2, False)
    opt = dict(irefatom=1, cutoff=6.0, dbulk=6.0, usecutoff=False, n_random_samples=5, **COMMON)
    compare(cm, orc, ms=30, aps=4, mv=200, apv=3, xs=xs, xv=xv, cells=cells, self_mode=False, precision="fp32",
            regime=regime, cell_scale_pct=pct, **opt)


@pytest.mark.parametrize("sched", ["cell", "balanced"])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("self_mode", [False, True], ids=["cross", "self"])
def test_atoms_schedules_match_oracle(cm, orc, gpu_ready, sched, precision, self_mode):
    """Both ATOMS evaluation schedules, forced whatever the solute density,
    give the oracle's counts (triclinic cell, custom groups, a cell size that
    widens the stencil beyond 27 cells)."""
    rng = np.random.default_rng(23 + self_mode)
    if self_mode:
        xs, xv, cells = make_system(rng, TRICLINIC, 12, 40, 12, 40, 2, True, spread=2.5)
        dims = dict(ms=12, aps=40, mv=12, apv=40)
    else:
        xs, xv, cells = make_system(rng, TRICLINIC, 2, 90, 300, 3, 2, False, spread=3.0)
        dims = dict(ms=2, aps=90, mv=300, apv=3)
    opt = dict(irefatom=2, cutoff=6.0, dbulk=6.0, usecutoff=False, n_random_samples=5, **COMMON)
    for pct in (0, 50):
        compare(cm, orc, xs=xs, xv=xv, cells=cells, self_mode=self_mode, precision=precision, regime="atoms",
                groups="custom", cell_scale_pct=pct, atoms_schedule=sched, **dims, **opt)


def test_autotune_reports_candidates(cm, gpu_ready):
    rng = np.random.default_rng(22)
    xs, xv, cells = make_system(rng, ORTHO, 200, 5, 200, 5, 3, True)
    t = cm.autotune(xs, None, cells, solute_nmols=200, solute_natomspermol=5, solvent_nmols=200,
                    solvent_natomspermol=5, autocorrelation=True, irefatom=1, cutoff=7.0, binstep=0.02, dbulk=7.0,
                    usecutoff=False, nbins=350, n_random_samples=4)
    # self-MDDF in the molecule layout: 4 cell sizes x both real-pass schedules
    ms = {(c["cell_scale_pct"], c["real_pass"]): c["ms_per_frame"] for c in t["candidates"]}
    assert len(ms) == 8 and all(v > 0 for v in ms.values()) and t["atoms_schedule"] == "auto"
    assert {k[1] for k in ms} == {"tile", "warp"}
    assert ms[(t["cell_scale_pct"], t["real_pass"])] == min(ms.values())


def test_autotune_atoms_tries_both_schedules(cm, gpu_ready):
    # the walk for every query (no candidate grid): both evaluation schedules
    rng = np.random.default_rng(24)
    xs, xv, cells = make_system(rng, ORTHO, 1, 120, 400, 3, 2, False, spread=3.0)
    t = cm.autotune(xs, xv, cells, solute_nmols=1, solute_natomspermol=120, solvent_nmols=400, solvent_natomspermol=3,
                    autocorrelation=False, irefatom=1, cutoff=7.0, binstep=0.02, dbulk=7.0, usecutoff=False,
                    nbins=350, n_random_samples=4, atoms_grid=-1)
    assert len(t["candidates"]) == 8
    assert {c["atoms_schedule"] for c in t["candidates"]} == {"cell", "balanced"}
    best = min(t["candidates"], key=lambda c: c["ms_per_frame"])
    assert (best["cell_scale_pct"], best["atoms_schedule"]) == (t["cell_scale_pct"], t["atoms_schedule"])


def test_autotune_atoms_grid_subdivisions(cm, gpu_ready):
    # one solute molecule in FP32: the walk (both schedules, two cell sizes) and the candidate grid
    rng = np.random.default_rng(25)
    xs, xv, cells = make_system(rng, ORTHO, 1, 120, 400, 3, 2, False, spread=3.0)
    t = cm.autotune(xs, xv, cells, solute_nmols=1, solute_natomspermol=120, solvent_nmols=400, solvent_natomspermol=3,
                    autocorrelation=False, irefatom=1, cutoff=7.0, binstep=0.02, dbulk=7.0, usecutoff=False,
                    nbins=350, n_random_samples=4, precision="fp32")
    assert len(t["candidates"]) == 8
    assert [(c["cell_scale_pct"], c["atoms_grid"]) for c in t["candidates"]] == [
        (100, -1), (100, -1), (80, -1), (80, -1), (100, 2), (100, 3), (100, 4), (100, 5)]
    assert {c["atoms_schedule"] for c in t["candidates"][:4]} == {"cell", "balanced"}
    best = min(t["candidates"], key=lambda c: c["ms_per_frame"])
    assert (best["cell_scale_pct"], best["atoms_grid"]) == (t["cell_scale_pct"], t["atoms_grid"])
