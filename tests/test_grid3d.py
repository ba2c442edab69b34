"""grid3D (src/tools/grid3D.jl:47-152): the CPU restatement against a
plain loop over points and atoms, the reference's argument error, the PDB
output, and -- on the GPU -- cm_grid3d against the restatement, point for
point and bit for bit."""
import math

import numpy as np
import pytest

from helpers import golden


def loop_grid3d(x, atype, table, d, dmin, dmax, step):
    """The reference's loops, one point and one atom at a time."""
    xmin, xmax = x.min(axis=0), x.max(axis=0)
    n = [int(math.ceil((xmax[k] - xmin[k] + 2 * dmax) / step + 1)) for k in range(3)]
    out = []
    for ix in range(1, n[0] + 1):
        for iy in range(1, n[1] + 1):
            for iz in range(1, n[2] + 1):
                p = (xmin[0] - dmax + step * (ix - 1), xmin[1] - dmax + step * (iy - 1), xmin[2] - dmax + step * (iz - 1))
                best, iat = math.inf, -1
                for a in range(len(x)):
                    # the norm of the displacement as a sum of abs2 (x * x) terms
                    e = [p[k] - x[a, k] for k in range(3)]
                    dd = e[0] * e[0] + e[1] * e[1] + e[2] * e[2]
                    if dd < best:
                        best, iat = dd, a
                r = math.sqrt(best)
                if dmin < r < dmax:
                    c = table[atype[iat]]
                    ir = next(i for i in range(len(d)) if d[i] > r)
                    il = ir - 1
                    cr = c[il] + (c[ir] - c[il]) / (d[ir] - d[il]) * (r - d[il])
                    if cr > 0:
                        out.append(((ix - 1) * n[1] * n[2] + (iy - 1) * n[2] + (iz - 1), iat, r, cr))
    return out


def test_restatement_matches_plain_loops(orc):
    rng = np.random.default_rng(3)
    x = rng.random((7, 3)) * 4.0
    atype = np.arange(7) % 3
    d = np.array([((0.5 * ((i * 0.1 + 0.1) ** 3 + (i * 0.1) ** 3)) ** (1 / 3)) for i in range(80)])
    table = rng.normal(size=(3, 80))
    got = orc.grid3d(x, atype, table, d, dmin=1.0, dmax=2.5, step=0.7)
    want = loop_grid3d(x, atype, table, d, 1.0, 2.5, 0.7)
    assert len(want) > 10
    assert [int(v) for v in got["point"]] == [w[0] for w in want]
    assert [int(v) for v in got["atom"]] == [w[1] for w in want]
    assert np.array_equal(got["distance"], np.array([w[2] for w in want]))
    assert np.array_equal(got["value"], np.array([w[3] for w in want]))


def namd_result(cm, nsolute=200):
    """The first residues of the NAMD fixture's protein against its 2,000 waters."""
    g = golden("namd_frames.npz")
    cells = np.array([np.diag([c[0], c[2], c[5]]) for c in g["cells"]])
    solute = cm.AtomSelection.from_indices(list(range(1, nsolute + 1)), nmols=1)
    water = cm.AtomSelection.from_indices(list(range(4013, 10013)), natomspermol=3)
    xw = np.repeat(g["water"].astype(np.float64)[None], 2, axis=0)
    tr = cm.ArrayTrajectory(solute, water, solute_frames=g["protein"][:, :nsolute].astype(np.float64),
                            solvent_frames=xw, cells=cells)
    return g, tr


def test_custom_groups_are_rejected(cm):
    sel = cm.AtomSelection.from_indices(list(range(1, 5)), nmols=1, group_atom_indices=[[1, 2], [3, 4]])
    R = cm.Result(nbins=10, dbulk=8.0, cutoff=8.0, autocorrelation=False, solute=sel, solvent=sel, files=[],
                  weights=[1.0])
    with pytest.raises(ValueError):
        cm.grid3D(R, cm.Atoms(np.zeros((4, 3))))


def test_pdb_output_reads_back(cm, tmp_path):
    g = cm.Grid3D(np.array([1.0, 2.5]), np.array([0.0, -3.25]), np.array([10.0, 11.0]), np.array([3, 7]),
                  np.array([1.75, 2.0]), np.array([0.2, 0.4]), np.array([0.0, 1.0]), ["OG1", "N"], ["THR", "GLY"],
                  ["A", "B"], [5, 12], ["O", "N"], (2, 2, 2), np.zeros(3))
    p = str(tmp_path / "g.pdb")
    g.write_pdb(p)
    a = cm.read_pdb_atoms(p)
    assert np.allclose(a.xyz, np.stack([g.x, g.y, g.z], axis=1), atol=1e-3)
    assert a.name == g.name and a.resname == g.resname and a.chain == g.chain and a.resnum == g.resnum


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["mddf", "coordination_number", "md_count"])
def test_gpu_grid3d_matches_restatement(cm, orc, gpu_ready, kind):
    g, tr = namd_result(cm)
    opts = cm.make_options(dbulk=10.0, n_random_samples=30, seed=4, silent=True)
    R = cm.mddf(tr, opts, coordination_number_only=(kind == "coordination_number"))
    atoms = cm.Atoms(g["protein"][0].astype(np.float64))
    G = cm.grid3D(R, atoms, dmin=1.5, dmax=5.0, step=0.5, type=kind)
    idx = np.asarray(R.solute.indices)
    table = cm.grid3d.atom_contribution_table(R, kind)
    ref = orc.grid3d(atoms.xyz[idx - 1], (idx - idx[0]) % R.solute.natomspermol, table, R.d, dmin=1.5, dmax=5.0,
                     step=0.5)
    assert len(G) == len(ref["point"]) > 100
    assert G.n == tuple(ref["n"])
    n = G.n
    assert np.array_equal(G.x, ref["origin"][0] + 0.5 * (ref["point"] // (n[1] * n[2])).astype(float))
    assert np.array_equal(G.index, idx[ref["atom"]])
    assert np.array_equal(G.occup, ref["distance"])
    assert np.array_equal(G.value, ref["value"])
    assert G.beta.min() == 0.0 and G.beta.max() == 1.0


@pytest.mark.parametrize("kind", ["mddf", "coordination_number", "md_count"])
def test_contribution_table_equals_one_atom_contributions(cm, orc, kind):
    """The vectorised table equals contributions() of each one-atom group."""
    g, tr = namd_result(cm, nsolute=30)
    from helpers import oracle_mddf

    R = oracle_mddf(cm, orc, tr, cm.make_options(dbulk=10.0, n_random_samples=5, seed=4, silent=True),
                    backend="cells")
    table = cm.grid3d.atom_contribution_table(R, kind)
    for t in range(R.solute.natomspermol):
        want = cm.contributions(R, cm.SoluteGroup([R.solute.indices[0] + t]), type=kind, _warn_zero_md_count=False)
        assert np.array_equal(table[t], want), t


# ------------------------------------------------------- a case solved by hand
# Two solute atoms, A at the origin (type 0) and B at (4, 0, 0) (type 1), a
# grid of step 1 with dmin = 1.5 and dmax = 2.5.  The grid spans the atoms'
# box widened by dmax: n = (10, 6, 6) points from (-2.5, -2.5, -2.5), so every
# coordinate of a point is a half-integer and twice a displacement from A or B
# is a triple of odd integers (a, b, c); the squared distance is
# (a^2 + b^2 + c^2) / 4.  No point is as close to A as to B (that needs
# x = 2, not a half-integer).  Sums of three odd squares
# between 4 dmin^2 = 9 and 4 dmax^2 = 25 are 11 and 19 only, so the kept
# points are the 24 permutations and sign patterns of (1, 1, 3) and the 24 of
# (1, 3, 3) around each atom: 96 points, at distances sqrt(11)/2 and
# sqrt(19)/2.  The contribution curves are c_A(d) = d and c_B(d) = 2 d, whose
# linear interpolation is the distance itself (A) or twice it (B).
HAND_XYZ = np.array([[0.0, 0.0, 0.0], [4.0, 0.0, 0.0]])
HAND_TYPE = np.array([0, 1])
HAND_D = np.arange(1, 61) * 0.05
HAND_TABLE = np.stack([HAND_D, 2.0 * HAND_D])


def hand_grid():
    """The kept points of the case above from integer arithmetic, in grid order:
    (linear index, closest atom, 4 x the squared distance)."""
    n = (10, 6, 6)
    out = []
    for ix in range(n[0]):
        for iy in range(n[1]):
            for iz in range(n[2]):
                b, c = 2 * iy - 5, 2 * iz - 5
                s_a, s_b = (2 * ix - 5) ** 2 + b * b + c * c, (2 * ix - 13) ** 2 + b * b + c * c
                atom, s = (0, s_a) if s_a < s_b else (1, s_b)
                if 9 < s < 25:
                    out.append(((ix * n[1] + iy) * n[2] + iz, atom, s))
    return n, out


def check_hand(point, atom, dist, val, n, origin):
    n_hand, want = hand_grid()
    assert len(want) == 96 and sorted({s for _, _, s in want}) == [11, 19]
    assert tuple(n) == n_hand and np.array_equal(np.asarray(origin), [-2.5, -2.5, -2.5])
    assert [int(p) for p in point] == [w[0] for w in want]
    assert [int(a) for a in atom] == [w[1] for w in want]
    r = np.array([math.sqrt(s) / 2.0 for _, _, s in want])
    assert np.array_equal(np.asarray(dist), r)
    assert np.allclose(val, r * np.array([1.0 + w[1] for w in want]), rtol=1e-14, atol=0.0)


def test_restatement_matches_the_case_solved_by_hand(orc):
    g = orc.grid3d(HAND_XYZ, HAND_TYPE, HAND_TABLE, HAND_D, dmin=1.5, dmax=2.5, step=1.0)
    check_hand(g["point"], g["atom"], g["distance"], g["value"], g["n"], g["origin"])


@pytest.mark.gpu
def test_gpu_grid3d_matches_the_case_solved_by_hand(cm, gpu_ready):
    check_hand(*cm.grid3d.grid_search(HAND_XYZ, HAND_TYPE, HAND_TABLE, HAND_D, dmin=1.5, dmax=2.5, step=1.0))
