"""GB300-native engine for the per-frame hot path of ComplexMixtures.jl.

The host-side API mirrors the reference's: ``Options``, ``AtomSelection``,
``Trajectory`` readers, ``mddf`` / ``coordination_number`` returning a
``Result``, and the ``contributions`` queries with ``SoluteGroup`` /
``SolventGroup``.  The per-frame minimum-distance search, histogramming and
random-insertion reference run in libcmgpu.so (CUDA, sm_103a) through the C
ABI of include/cmgpu.h; there is no CPU fallback.
"""
from .options import Options, TrajectoryFileOptions, make_options
from .selection import (AtomSelection, SoluteGroup, SolventGroup, atom_group, atom_group_name,
                        atom_group_names, set_nmols_natomspermol)
from .results import (Density, Result, Volume, finalresults, load, merge, renormalize, result_from_json, save, setbin,
                      shellradius, snapshot_from_result, sphericalshellvolume, sum_results, units)
from .trajectory import (ArrayTrajectory, NamdDCD, PDBTraj, Trajectory, TrajectoryMetaData, convert_unitcell,
                         make_trajectory, trajectory_metadata, unitcell_from_lengths_angles)
from .contributions import ResidueContributions, contribution_terms, contributions
from .engine import Batch, Engine, autotune, load_snapshot, memory_cache, save_snapshot
from .grid3d import Atoms, Grid3D, grid3D, read_pdb_atoms
from .server import Server, latency_percentiles
from .mddf import coordination_number, engine_for, mddf, new_result
from ._native import NativeUnavailable

__all__ = [
    "Options", "TrajectoryFileOptions", "make_options", "AtomSelection", "SoluteGroup", "SolventGroup",
    "atom_group", "atom_group_name", "atom_group_names", "set_nmols_natomspermol", "Density", "Result",
    "Volume", "finalresults", "renormalize", "result_from_json", "setbin", "shellradius", "sphericalshellvolume",
    "sum_results", "units", "save", "load", "merge", "snapshot_from_result", "save_snapshot", "load_snapshot", "ArrayTrajectory", "NamdDCD", "PDBTraj", "Trajectory", "TrajectoryMetaData",
    "convert_unitcell", "make_trajectory", "trajectory_metadata", "unitcell_from_lengths_angles", "contributions", "contribution_terms", "ResidueContributions",
    "Atoms", "Grid3D", "grid3D", "read_pdb_atoms", "Batch", "Engine", "autotune", "memory_cache", "Server", "latency_percentiles", "coordination_number", "engine_for", "mddf", "new_result", "NativeUnavailable",
]
