"""Extract the golden fixtures used by the tests from ComplexMixtures.jl's own
test data (run once in a checkout that has the reference next to it):

    python tests/golden/make_fixtures.py /path/to/ComplexMixtures.jl

Writes, next to this script:
  toy.npz            coordinates and cells of test/data/toy/{cross,self_monoatomic,
                     self_monoatomic_duplicated_first_frame}.pdb
  namd_frames.npz    frames 1 and 3 of test/data/NAMD/traj_duplicated_first_frame.dcd
                     (frame 3 is frame 2 of NAMD/trajectory.dcd) for the protein
                     (atoms 1-1463) and TMAO (1479-4012), frame 1 for the first
                     2,000 waters (4013-10012), and the TMAO atom names
  json_<name>.npz    fields of the saved Results test/data/{NAMD,Gromacs,PDB}/*.json

The files are read, never modified; the tests only read the .npz files.
"""
from __future__ import annotations

import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_pdb(path):
    frames, cells, cur, cell = [], [], [], None
    with open(path) as f:
        for line in f:
            if line.startswith("CRYST1"):
                t = line.split()
                cell = [float(t[1]), float(t[2]), float(t[3])]
            elif line.startswith(("ATOM", "HETATM")):
                cur.append((float(line[30:38]), float(line[38:46]), float(line[46:54])))
            elif line.startswith("END"):
                if cur:
                    frames.append(cur)
                    cells.append(cell)
                cur = []
    if cur:
        frames.append(cur)
        cells.append(cell)
    return np.array(frames), np.array(cells)


def read_dcd(path):
    data = open(path, "rb").read()
    off = 0

    def rec():
        nonlocal off
        (n,) = struct.unpack_from("<i", data, off)
        out = data[off + 4 : off + 4 + n]
        off += 8 + n
        return out

    rec(), rec()
    (natoms,) = struct.unpack("<i", rec())
    frames, cells = [], []
    while off < len(data):
        uc = struct.unpack("<6d", rec())
        x = np.frombuffer(rec(), "<f4")
        y = np.frombuffer(rec(), "<f4")
        z = np.frombuffer(rec(), "<f4")
        frames.append(np.stack([x, y, z], axis=1))
        cells.append(uc)
    return np.array(frames), np.array(cells), natoms


def main(ref):
    d = os.path.join(ref, "test", "data")
    out = {}
    for name in ("cross", "self_monoatomic", "self_monoatomic_duplicated_first_frame"):
        x, c = parse_pdb(os.path.join(d, "toy", name + ".pdb"))
        out[name + "_xyz"] = x
        out[name + "_cell"] = c
    np.savez_compressed(os.path.join(HERE, "toy.npz"), **out)

    frames, cells, natoms = read_dcd(os.path.join(d, "NAMD", "traj_duplicated_first_frame.dcd"))
    tm = json.load(open(os.path.join(d, "NAMD", "tmao_tmao.json")))
    np.savez_compressed(
        os.path.join(HERE, "namd_frames.npz"),
        protein=frames[[0, 2], 0:1463],
        tmao=frames[[0, 2], 1478:4012],
        water=frames[0, 4012 : 4012 + 6000],
        cells=cells[[0, 2]],
        natoms=natoms,
        tmao_names=np.array(tm["solute"]["group_names"]),
    )

    for sub, name in (("NAMD", "tmao_tmao"), ("NAMD", "water_tmao"), ("NAMD", "water_water"), ("Gromacs", "EMI_DCA"),
                      ("Gromacs", "EMI_EMI"), ("PDB", "tmao_tmao")):
        D = json.load(open(os.path.join(d, sub, name + ".json")))
        o = D["files"][0]["options"]
        rec_ = {
            "nbins": D["nbins"], "dbulk": D["dbulk"], "cutoff": D["cutoff"], "autocorrelation": D["autocorrelation"],
            "binstep": o["binstep"], "usecutoff": o["usecutoff"], "n_random_samples": o["n_random_samples"],
            "firstframe": o["firstframe"], "stride": o["stride"], "lastframe_read": D["files"][0]["lastframe_read"],
            "frame_weights": np.array(D["files"][0]["frame_weights"], dtype=np.float64),
            "solute_nmols": D["solute"]["nmols"], "solute_natomspermol": D["solute"]["natomspermol"],
            "solvent_nmols": D["solvent"]["nmols"], "solvent_natomspermol": D["solvent"]["natomspermol"],
            "solute_first_index": D["solute"]["indices"][0], "solvent_first_index": D["solvent"]["indices"][0],
            "solute_group_names": np.array(D["solute"]["group_names"]),
            "solvent_group_names": np.array(D["solvent"]["group_names"]),
            "volume_total": D["volume"]["total"], "volume_bulk": D["volume"]["bulk"],
            "volume_domain": D["volume"]["domain"], "volume_shell": np.array(D["volume"]["shell"]),
            "density_solute": D["density"]["solute"], "density_solvent": D["density"]["solvent"],
            "density_solvent_bulk": D["density"]["solvent_bulk"],
        }
        for k in ("d", "md_count", "md_count_random", "coordination_number", "coordination_number_random", "mddf", "kb",
                  "rdf_count", "rdf_count_random", "sum_rdf_count", "sum_rdf_count_random", "rdf", "kb_rdf"):
            rec_[k] = np.array(D[k], dtype=np.float64)
        for k in ("solute_group_count", "solvent_group_count", "solute_group_count_random", "solvent_group_count_random"):
            rec_[k] = np.array(D[k], dtype=np.float64)
        tag = f"json_{sub.lower()}_{name}.npz"
        np.savez_compressed(os.path.join(HERE, tag), **rec_)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_fixtures.py <path of a ComplexMixtures.jl checkout>")
    main(sys.argv[1])
