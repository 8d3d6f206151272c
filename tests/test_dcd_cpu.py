"""The DCD restatement against the reference's own writer (src/dcdio.cpp,
built from the reference tree into oracle/_ref when the tree is present)."""
import os
import subprocess

import numpy as np
import pytest

from oracle import dcd_oracle as D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DCD = os.path.join(ROOT, "oracle", "_ref", "ref_dcd")


@pytest.mark.skipif(not os.path.exists(REF_DCD), reason="the reference tree was not available to build oracle/_ref")
def test_dcd_bytes_match_reference_writer(tmp_path):
    rng = np.random.default_rng(5)
    N, F = 37, 4
    frames = rng.normal(size=(F, 3, N)).astype(np.float32) * 50
    src = tmp_path / "frames.bin"
    src.write_bytes(frames.tobytes())
    out = tmp_path / "ref.dcd"
    subprocess.run([REF_DCD, str(out), str(N), "25", "1", "1000", "100.0", str(src)], check=True)
    mine = D.header(N, 25, 1, 1000, 100.0, "REMARKS FIXED FOR COMPARISON")
    for f in frames:
        mine += D.frame(f[0], f[1], f[2])
    assert out.read_bytes() == mine


def test_dcd_layout():
    h = D.header(10, 5, 1, 100, 0.5, "R")
    assert len(h) == 4 + 84 + 4 + 4 + 164 + 4 + 4 + 4 + 4
    fr = D.frame(np.zeros(10), np.ones(10), np.arange(10))
    assert len(fr) == 3 * (4 + 40 + 4)


def test_reader_reads_reference_writer_output(tmp_path):
    from mt_gb300 import dcd
    rng = np.random.default_rng(6)
    N, F = 21, 3
    fx = rng.normal(size=(F, 3, N)).astype(np.float32)
    fa = rng.normal(size=(F, 3, N)).astype(np.float32)
    xyz, ang = tmp_path / "x.dcd", tmp_path / "a.dcd"
    if os.path.exists(REF_DCD):
        for frames, out in ((fx, xyz), (fa, ang)):
            src = tmp_path / "f.bin"
            src.write_bytes(frames.tobytes())
            subprocess.run([REF_DCD, str(out), str(N), str(F), "1", "10", "100.0", str(src)], check=True)
    else:
        for frames, out in ((fx, xyz), (fa, ang)):
            b = D.header(N, F, 1, 10, 100.0, "R")
            for f in frames:
                b += D.frame(f[0], f[1], f[2])
            out.write_bytes(b)
    got = list(dcd.read_frames(str(xyz), str(ang)))
    assert len(got) == F
    for k in range(F):
        np.testing.assert_array_equal(got[k][:, 0:3], fx[k].T)
        np.testing.assert_array_equal(got[k][:, 3], fa[k][0])   # fi
        np.testing.assert_array_equal(got[k][:, 5], fa[k][1])   # psi
        np.testing.assert_array_equal(got[k][:, 4], fa[k][2])   # theta
