"""DCD frames read as raw bytes and decoded on the device (cm_set_dcd_layout +
CM_COORD_DCD): the raw reader against the record-by-record reader
(src/trajectory_formats/NamdDCD.jl:141-188) on files written here in both byte
orders, and -- on the GPU -- mddf through the device decode against mddf on
the same float32 coordinates gathered on the host, and against the oracle."""
import struct

import numpy as np
import pytest

from helpers import golden, oracle_mddf


def write_dcd(path, frames, cells6, endian="<"):
    """A NAMD-style DCD: header, title and natoms records, then per frame the
    unit-cell record (A, gamma, B, beta, alpha, C) and the x, y, z records."""
    n, natoms, _ = frames.shape

    def rec(b):
        return struct.pack(endian + "i", len(b)) + b + struct.pack(endian + "i", len(b))

    hdr = b"CORD" + struct.pack(endian + "9i", n, 1, 1, n, 0, 0, 0, 0, 0) + struct.pack(endian + "f", 0.0) + \
        struct.pack(endian + "10i", 1, 0, 0, 0, 0, 0, 0, 0, 0, 24)
    with open(path, "wb") as f:
        f.write(rec(hdr))
        f.write(rec(struct.pack(endian + "i", 1) + b"written by the test suite".ljust(80)))
        f.write(rec(struct.pack(endian + "i", natoms)))
        for k in range(n):
            f.write(rec(np.asarray(cells6[k], dtype=endian + "f8").tobytes()))
            for ax in range(3):
                f.write(rec(np.ascontiguousarray(frames[k, :, ax], dtype=endian + "f4").tobytes()))


def namd_system(nframes=4):
    """Protein + TMAO + water frames from the reference's NAMD fixture, jittered
    to make more frames; cells in DCD order."""
    g = golden("namd_frames.npz")
    rng = np.random.default_rng(4)
    base = [np.concatenate([g["protein"][k], g["tmao"][k], g["water"]]) for k in range(2)]
    frames = np.stack([base[k % 2] + rng.normal(scale=0.05, size=base[0].shape) for k in range(nframes)])
    cells6 = np.stack([g["cells"][k % 2] for k in range(nframes)])
    return frames.astype(np.float32), cells6


def selections(cm):
    tmao = cm.AtomSelection.from_indices(list(range(1464, 1464 + 2534)), natomspermol=14)
    water = cm.AtomSelection.from_indices(list(range(3998, 3998 + 6000)), natomspermol=3)
    return tmao, water


@pytest.mark.parametrize("endian", ["<", ">"], ids=["little", "big"])
def test_raw_frames_match_record_reader(cm, tmp_path, endian):
    frames, cells6 = namd_system(3)
    path = str(tmp_path / "t.dcd")
    write_dcd(path, frames, cells6, endian)
    tmao, water = selections(cm)
    t = cm.NamdDCD(path, tmao, water)
    assert t.nframes == 3
    lay = t.dcd_layout()
    assert lay["big_endian"] == (endian == ">")
    raw, cells = t.read_raw(0, 3)
    assert raw.shape == (3, lay["frame_bytes"])
    t.opentraj()
    for k in range(3):
        t.nextframe()
        assert np.array_equal(cells[k], t.getunitcell())
        dt = np.dtype(endian + "f4")
        xyz = np.stack([np.frombuffer(raw[k, o:o + 4 * lay["natoms"]].tobytes(), dtype=dt)
                        for o in (lay["x_offset"], lay["y_offset"], lay["z_offset"])], axis=1)
        assert np.array_equal(xyz[np.asarray(tmao.indices) - 1], t.x_solute)
        assert np.array_equal(xyz[np.asarray(water.indices) - 1], t.x_solvent)
    t.closetraj()
    one, c1 = t.read_raw(2, 1)
    assert np.array_equal(one[0], raw[2]) and np.array_equal(c1[0], cells[2])


def test_raw_reader_rejects_corrupted_records(cm, tmp_path):
    frames, cells6 = namd_system(2)
    path = str(tmp_path / "bad.dcd")
    write_dcd(path, frames, cells6)
    tmao, water = selections(cm)
    t = cm.NamdDCD(path, tmao, water)
    with open(path, "r+b") as f:       # break the y record's end marker of frame 2
        lay = t.dcd_layout()
        f.seek(t._data_start + lay["frame_bytes"] + lay["y_offset"] + 4 * lay["natoms"])
        f.write(struct.pack("<i", 7))
    t.read_raw(0, 1)
    with pytest.raises(ValueError):
        t.read_raw(1, 1)
    with pytest.raises(ValueError):
        t.read_raw(1, 5)                 # past the end of the file


@pytest.mark.gpu
@pytest.mark.parametrize("endian", ["<", ">"], ids=["little", "big"])
@pytest.mark.parametrize("frames_kw", [dict(), dict(firstframe=2, stride=2)], ids=["all", "strided"])
def test_device_decode_mddf_matches_host_gather(cm, orc, gpu_ready, tmp_path, endian, frames_kw):
    frames, cells6 = namd_system(5)
    path = str(tmp_path / "t.dcd")
    write_dcd(path, frames, cells6, endian)
    tmao, water = selections(cm)
    opts = cm.make_options(dbulk=8.0, n_random_samples=3, seed=77, silent=True,
                           **frames_kw)
    Rd = cm.mddf(cm.NamdDCD(path, tmao, water), opts)             # raw frames, decoded on the device
    cells = np.stack([cm.NamdDCD._cell_of(c) for c in cells6])
    s = np.asarray(tmao.indices) - 1
    v = np.asarray(water.indices) - 1
    arr = cm.ArrayTrajectory(tmao, water, solute_frames=frames[:, s].astype(np.float64),
                             solvent_frames=frames[:, v].astype(np.float64), cells=cells)
    Rh = cm.mddf(arr, opts)                                       # host-gathered float64 coordinates
    for f in ("md_count", "md_count_random", "rdf_count", "rdf_count_random", "solute_group_count",
              "solvent_group_count", "mddf", "kb", "coordination_number"):
        assert np.array_equal(getattr(Rd, f), getattr(Rh, f)), f
    assert Rd.volume.total == Rh.volume.total
    Ro = oracle_mddf(cm, orc, cm.NamdDCD(path, tmao, water), opts, backend="cells")
    for f in ("md_count", "md_count_random", "rdf_count", "rdf_count_random", "mddf", "kb"):
        assert np.array_equal(getattr(Rd, f), getattr(Ro, f)), f
