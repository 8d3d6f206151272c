"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/mtg.h declares (no compute calls: these run without a GPU)."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(mtg_\w+)\s*\(", src))
    return names


def test_library_exports_header(engine_mod):
    out = subprocess.run(["nm", "-D", "--defined-only", engine_mod.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\b(mtg_\w+)\b", out))
    missing = declared_symbols() - exported
    assert not missing, missing
    # the Python binding declares every header entry point
    assert declared_symbols() <= set(engine_mod.EXPORTS)


def test_library_built_for_sm103a_only():
    """The build compiles every translation unit for sm_103a alone (no PTX
    for other targets, no multi-architecture fat binary); the GPU test
    test_device_code_is_sm103a checks the loaded code at run time."""
    from mt_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_derive_params_matches_reference_formula(engine_mod):
    from mt_gb300 import synth
    p = synth.default_params(seed=2)
    q = synth.default_params(seed=2)
    engine_mod.derive_params(q)
    for k in ("gammaR", "gammaTheta", "varR", "varTheta"):
        assert getattr(p, k) == getattr(q, k), k
    # hdi_on switches the translational radius to tea_a (src/preparator.cpp:209-213)
    q.hdi_on, q.tea_a = 1, 3.0
    engine_mod.derive_params(q)
    assert abs(q.gammaR - 6 * np.pi * q.viscosity * 3.0) / q.gammaR < 1e-6


def test_invalid_params_rejected_without_gpu(engine_mod):
    """Argument checks run before any CUDA call and return MTG_E_CONFIG with
    the reason."""
    import ctypes as C
    from mt_gb300 import _abi, synth
    lib = engine_mod.load()
    h = C.c_void_p()
    t = _abi.MtgTopology()                       # no beads
    rc = lib.mtg_create(C.byref(synth.default_params()), C.byref(t), C.byref(h))
    assert rc == _abi.MTG_E_CONFIG and b"Ntot > 0" in lib.mtg_last_error_string()
    t.Ntot, t.Ntr = 8, 1                         # beads but no topology arrays
    rc = lib.mtg_create(C.byref(synth.default_params()), C.byref(t), C.byref(h))
    assert rc == _abi.MTG_E_CONFIG and b"required" in lib.mtg_last_error_string()
    for over, word in ((dict(ljpairsupdatefreq=0), "ljpairsupdatefreq"),
                       (dict(hdi_on=1, tea_epsilon_freq=0), "tea_epsilon_freq")):   # the reference would divide by zero
        b = synth.uniform_batch(synth.default_params(**over), 1, 4, 2, seed=1)
        with pytest.raises(engine_mod.MtgError, match=word):
            engine_mod.Engine(b)


def test_empty_trajectory_rejected(engine_mod):
    """An empty trajectory is a configuration error (MTG_E_CONFIG), reported
    before any device work: the reference never has one."""
    from mt_gb300 import synth
    p = synth.default_params(seed=5)
    trajs = [synth.make_trajectory(6, 20, seed=5, radius=8.12, psi_mode="make_mt", cube=40.0),
             synth.make_trajectory(0, 0, seed=6, radius=8.12, psi_mode="make_mt", cube=40.0)]
    b = synth.batch_from_trajectories(p, trajs)
    with pytest.raises(engine_mod.MtgError, match="MTG_E_CONFIG"):
        engine_mod.Engine(b)


def test_kernel_kinds_match_header(engine_mod):
    """The Python names of the per-kernel timing kinds cover MTG_KERNEL_KINDS."""
    src = open(os.path.join(ROOT, "include", "mtg.h")).read()
    n = int(re.search(r"#define\s+MTG_KERNEL_KINDS\s+(\d+)", src).group(1))
    assert len(engine_mod.KERNEL_KINDS) == n
    assert len(set(engine_mod.KERNEL_KINDS)) == n
