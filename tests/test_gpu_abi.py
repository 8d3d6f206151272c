"""The library's device code on the GPU: the kernels that run are the sm_103a
build (checked at run time through cudaFuncGetAttributes, not by reading the
binary)."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def test_device_code_is_sm103a(engine_mod):
    lib = engine_mod.load()
    bv, pv = C.c_int(), C.c_int()
    engine_mod.check(lib.mtg_device_code_version(0, C.byref(bv), C.byref(pv)))
    assert bv.value == 103, bv.value
