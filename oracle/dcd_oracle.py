"""DCD writer/reader of the reference's dcdio.cpp restated in Python
(TEST INFRASTRUCTURE ONLY): dcdWriteHeader (src/dcdio.cpp:98-154, no unit
cell), dcdWriteFrame (:179-203) and the frame sequence of saveCoordDCD
(src/preparator.cpp:582-602): (x, y, z) in the coordinate file and
(fi, psi, theta) in the angle file."""
import struct

import numpy as np


def header(N, nfile, npriv, nsavc, delta, remark2, remark1="REMARKS CREATED BY dcdio.c"):
    b = struct.pack("<i4s4i5if9i", 84, b"CORD", nfile, npriv, nsavc, npriv - nsavc, 0, 0, 0, 0, 0,
                    np.float32(delta), 0, 0, 0, 0, 0, 0, 0, 0, 0)
    b += struct.pack("<4i", 24, 84, 164, 2)
    for r in (remark1, remark2):
        raw = r.encode()[:79]
        b += raw + b"\0" * (80 - len(raw))
    b += struct.pack("<4i", 164, 4, N, 4)
    return b


def frame(X, Y, Z):
    out = b""
    for a in (X, Y, Z):
        a = np.ascontiguousarray(a, np.float32)
        out += struct.pack("<i", 4 * len(a)) + a.tobytes() + struct.pack("<i", 4 * len(a))
    return out


def trajectory_files(states, offsets, nfile, npriv, nsavc, delta, remark2):
    """Bytes of the coordinate and angle DCD files of every trajectory for a
    sequence of Coord AoS states (x, y, z, fi, theta, psi, w)."""
    files = []
    for t in range(len(offsets) - 1):
        a, e = offsets[t], offsets[t + 1]
        xyz = header(e - a, nfile, npriv, nsavc, delta, remark2)
        ang = header(e - a, nfile, npriv, nsavc, delta, remark2)
        for s in states:
            c = np.asarray(s, np.float32)[a:e]
            xyz += frame(c[:, 0], c[:, 1], c[:, 2])
            ang += frame(c[:, 3], c[:, 5], c[:, 4])
        files.append((xyz, ang))
    return files
