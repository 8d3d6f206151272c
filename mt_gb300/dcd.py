"""DCD frames back into engine states: the re-analysis path.

Reads the coordinate and angle DCD files that the reference's saveCoordDCD
(src/preparator.cpp:582-602) and mtg_output_frame write (dcdWriteHeader /
dcdWriteFrame layout, src/dcdio.cpp:98-203, no unit cell) and rebuilds the
Coord AoS states (x, y, z, fi, theta, psi, w) frame by frame, as the
reference's READ_FROM_DCD build does (ReadFromDCD, src/preparator.cpp:635-662,
called from src/main.cpp:54-65).  `analyse` evaluates the energies of every
frame of a batch on the GPU.
"""
from __future__ import annotations

import struct

import numpy as np


def _read_header(f):
    b = f.read(4 + 84 + 4)
    if len(b) < 92 or struct.unpack("<i", b[:4])[0] != 84 or b[4:8] != b"CORD":
        raise ValueError("not a DCD file: no 84 / CORD header")
    nfile, npriv, nsavc = struct.unpack("<3i", b[8:20])
    has_uc = struct.unpack("<i", b[48:52])[0]
    (n164,) = struct.unpack("<i", f.read(4))
    f.read(n164 + 4)                                 # remarks block and its end marker
    n4, natoms, _ = struct.unpack("<3i", f.read(12))
    if n4 != 4:
        raise ValueError("unexpected DCD atom-count record")
    return {"nfile": nfile, "npriv": npriv, "nsavc": nsavc, "has_uc": has_uc, "natoms": natoms}


def _frames(path):
    with open(path, "rb") as f:
        h = _read_header(f)
        n = h["natoms"]
        while True:
            if h["has_uc"]:
                rec = f.read(4 + 48 + 4)
                if len(rec) < 56:
                    return
            out = []
            for _ in range(3):
                b = f.read(4 + 4 * n + 4)
                if len(b) < 8 + 4 * n:
                    return
                out.append(np.frombuffer(b[4:4 + 4 * n], np.float32))
            yield np.stack(out, 1)


def read_frames(xyz_path: str, ang_path: str):
    """Yields one Coord AoS array [n, 7] per frame of a trajectory's two DCD
    files: (x, y, z) from the coordinate file, (fi, psi, theta) from the
    angle file."""
    for xyz, ang in zip(_frames(xyz_path), _frames(ang_path)):
        c = np.zeros((len(xyz), 7), np.float32)
        c[:, 0:3] = xyz
        c[:, 3] = ang[:, 0]     # fi
        c[:, 5] = ang[:, 1]     # psi
        c[:, 4] = ang[:, 2]     # theta
        yield c


def read_batch(xyz_paths, ang_paths):
    """Frames of a batch (one pair of files per trajectory, in order):
    yields the concatenated Coord AoS state of all trajectories per frame."""
    gens = [read_frames(x, a) for x, a in zip(xyz_paths, ang_paths)]
    for parts in zip(*gens):
        yield np.concatenate(parts, 0)


def analyse(engine, xyz_paths, ang_paths):
    """Per-frame energy totals [frames, ntraj, 7] of a batch's DCD files:
    every frame is uploaded to the engine and evaluated on the GPU."""
    out = []
    for state in read_batch(xyz_paths, ang_paths):
        engine.upload_state(state)
        engine.rebuild_pairs()
        out.append(engine.energies())
    return np.array(out)
