"""The learned mode's far-field tree, built by the engine's own host code
(mt_gb300/csrc/tea_ff.cu compiled into tests/fftree/tree_check.cu with
nvcc, run on the CPU): every ordered bead pair of a trajectory is covered
exactly once by a near leaf pair or a far node pair, on trajectories of the
learned-TEA workload, on a small uneven batch, and with extra beads (which
stay out of the tree)."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


@pytest.fixture(scope="module")
def tree_check(tmp_path_factory):
    if not os.path.exists(NVCC):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("fftree") / "tree_check")
    src = os.path.join(ROOT, "tests", "fftree", "tree_check.cu")
    r = subprocess.run([NVCC, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "mt_gb300", "csrc"), src, "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return out


def dump(b, path):
    flags = (b.extra != 0).astype(np.int32)          # the extra-bead flag bit
    x = np.zeros((b.nbeads, 4), np.float32)
    x[:, :3] = b.coords[:, :3]
    with open(path, "wb") as f:
        np.array([b.nbeads, b.ntraj], np.int32).tofile(f)
        np.asarray(b.offsets, np.int32).tofile(f)
        flags.tofile(f)
        x.tofile(f)


def run(exe, path, theta, ntraj):
    r = subprocess.run([exe, path, str(theta), str(ntraj)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_tree_of_learned_workload(tree_check, tmp_path):
    import bench
    b = bench.make_batch(dict(bench.WORKLOADS["tea_exact_64x5600"]), 1, 2)
    p = str(tmp_path / "b.bin")
    dump(b, p)
    for theta in (0.85, 1.0):
        out = run(tree_check, p, theta, 2)
        assert "bad 0" in out, out


def test_tree_of_uneven_batch(tree_check, tmp_path):
    from mt_gb300 import synth
    pr = synth.default_params(seed=3, hdi_on=1)
    b = synth.ragged_batch(pr, 5, seed=3, pf_range=(2, 30), free_range=(0, 400), cube=80.0)
    p = str(tmp_path / "b.bin")
    dump(b, p)
    out = run(tree_check, p, 0.85, 5)
    assert "bad 0" in out, out


def test_tree_leaves_out_extra_beads(tree_check, tmp_path):
    from mt_gb300 import synth
    pr = synth.default_params(seed=4, hdi_on=1)
    b = synth.uniform_batch(pr, 2, 20, 300, seed=4, cube=60.0, n_extra_dimers=3)
    assert b.extra.sum() > 0
    p = str(tmp_path / "b.bin")
    dump(b, p)
    out = run(tree_check, p, 0.85, 2)
    assert "bad 0" in out, out
