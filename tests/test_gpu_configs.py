"""Parity at the shapes of the five benchmark configurations: the engine's
int64 half-unit counts equal the oracle's, bit for bit, on the seeded
synthetic systems of each configuration (full size where the oracle takes
seconds, a few frames each).

  c1  1,200-atom chain in 5,000 waters, 10 frames, groups of 10 (ATOMS layout)
  c2  20,000-atom confined chain with 50,000 waters and 2,000 14-atom
      cosolvent molecules: two MDDFs per frame (ATOMS layout), FP32 frames
  c3  10,000 rigid 14-atom molecules, self-MDDF, triclinic cell (PAIRS layout)
  c4  systems of 2,064 / 21,000 / 183,750 atoms: 5 % chain + water
  c5  c3-like requests with cutoffs drawn in [8, 14]
"""
import importlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("md", "md_random", "rdf", "rdf_random", "solute_group", "solute_group_random", "solvent_group",
        "solvent_group_random")


def syn():
    return importlib.import_module("complexmixtures_gb300.synth")


def run_both(cm, orc, sysm, nframes, solvent=0, precision="fp32", frames=None):
    xs, xv, cells = sysm.frames(nframes, solvent=solvent) if frames is None else frames
    self_mode = sysm.self_mddf
    sv = None if self_mode else sysm.solvents[solvent]
    aps, ms = sysm.solute_natomspermol, sysm.solute_nmols
    mv, apv = (ms, aps) if self_mode else (sv.nmols, sv.natomspermol)
    g = {}
    if sysm.solute_group_size:
        size = sysm.solute_group_size
        g = dict(solute_groups=[[i // size] for i in range(aps)], solute_ngroups=(aps + size - 1) // size)
    kw = dict(autocorrelation=self_mode, irefatom=1, cutoff=sysm.cutoff, binstep=sysm.binstep, dbulk=sysm.cutoff,
              usecutoff=False, nbins=cm.setbin(sysm.cutoff, sysm.binstep), n_random_samples=sysm.n_random_samples,
              seed=sysm.seed, **g)
    ids = np.arange(1, nframes + 1)
    eng = cm.Engine(solute_nmols=ms, solute_natomspermol=aps, solvent_nmols=mv, solvent_natomspermol=apv,
                    precision=precision, **kw)
    eng.submit(xs, xv, cells, frame_ids=ids)
    got = eng.raw_counts()
    st = eng.stats()
    eng.close()
    ref = orc.run(ms=ms, aps=aps, mv=mv, apv=apv, solute_xyz=xs.astype(np.float64),
                  solvent_xyz=None if self_mode else xv.astype(np.float64), cells=cells, frame_ids=ids,
                  nthreads=os.cpu_count() or 1, **kw)
    for k in KEYS:
        if self_mode and k.startswith("solvent"):
            continue
        assert np.array_equal(got[k], ref[k]), (sysm.name, k, np.nonzero(got[k] != ref[k]))
    assert ref["md"].sum() > 0 and ref["md_random"].sum() > 0
    return st


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_config1(cm, orc, gpu_ready, precision):
    st = run_both(cm, orc, syn().config1(), 10, precision=precision)
    assert st["regime"] == cm._native.CM_REGIME_ATOMS


@pytest.mark.parametrize("solvent", [0, 1], ids=["water", "cosolvent"])
def test_config2(cm, orc, gpu_ready, solvent):
    run_both(cm, orc, syn().config2(), 2, solvent=solvent)


def test_config3(cm, orc, gpu_ready):
    s = syn().config3(nframes=2)
    st = run_both(cm, orc, s, 2)
    assert st["regime"] == cm._native.CM_REGIME_PAIRS


@pytest.mark.parametrize("natoms", [2064, 21000, 183750])
def test_config4(cm, orc, gpu_ready, natoms):
    run_both(cm, orc, syn().config4_system(natoms, 20261207 + natoms, nframes=2), 2)


@pytest.mark.parametrize("natoms", [5000, 60000])
def test_config5(cm, orc, gpu_ready, natoms):
    s = syn().config5_request(natoms, 20261208 + natoms, 3)
    assert 8.0 <= s.cutoff <= 14.0
    run_both(cm, orc, s, 3)
