"""mtg_energies_noalloc: per-trajectory energy totals computed without any
allocation, for callers that must not allocate device memory when they ask
for energies (hooks running next to in-flight work on the same GPU, where
cudaMalloc/cudaFree could synchronise the device; pool-managed processes
where a new cudaMalloc could fail).  Checked through the C ABI against the
allocating entry point mtg_energies, on two calls in a row (the fixed scratch
is reused) with a different state for each call."""
import ctypes as C

import numpy as np
import pytest

from helpers import small_system

pytestmark = pytest.mark.gpu


def test_noalloc_totals_match_mtg_energies(engine_mod):
    import torch

    b = small_system(seed=21, ntr=3)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.rebuild_pairs()
    lib = engine_mod.load()
    out = torch.empty(b.ntraj * 7, dtype=torch.float64, device="cuda:0")
    for call in range(2):
        expected = e.energies()                       # allocating path, host totals
        out.fill_(float("nan"))                       # stale results would show as NaN
        torch.cuda.synchronize()
        rc = lib.mtg_energies_noalloc(e.h, C.c_void_p(out.data_ptr()))
        assert rc == 0, lib.mtg_last_error_string().decode()
        engine_mod.check(lib.mtg_sync(e.h))
        got = out.cpu().numpy().reshape(b.ntraj, 7)
        np.testing.assert_allclose(got, expected, rtol=1e-12, atol=1e-12)
        e.step(10 * call, 10)                         # the second call sees a new state
    e.close()


def test_noalloc_calls_allocate_nothing(engine_mod):
    """After a first call (which looks up the scratch address), further calls
    leave the device's free memory unchanged: the property the entry point
    exists for."""
    import torch

    b = small_system(seed=22, ntr=2)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.rebuild_pairs()
    lib = engine_mod.load()
    out = torch.empty(b.ntraj * 7, dtype=torch.float64, device="cuda:0")
    assert lib.mtg_energies_noalloc(e.h, C.c_void_p(out.data_ptr())) == 0
    engine_mod.check(lib.mtg_sync(e.h))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(20):
        assert lib.mtg_energies_noalloc(e.h, C.c_void_p(out.data_ptr())) == 0
    engine_mod.check(lib.mtg_sync(e.h))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)
    e.close()


def test_noalloc_rejects_oversized_batch(engine_mod):
    """More chunks than the fixed scratch holds -> MTG_E_CONFIG with a message."""
    from mt_gb300 import synth

    ntraj = 16385                                     # one 128-bead chunk per trajectory
    p = synth.default_params(seed=1, is_assembly=0, lj_on=0)
    n = 2 * ntraj
    b = synth.Batch(params=p, offsets=(2 * np.arange(ntraj + 1)).astype(np.int32),
                    coords=np.zeros((n, 7), np.float32), mon_type=np.tile(np.array([0, 1], np.int32), ntraj),
                    fixed=np.zeros(n, np.uint8), extra=np.zeros(n, np.uint8), gtp=np.ones(n, np.int32),
                    on_tubule=np.zeros(n, np.int32), harmonic_count=np.ones(n, np.int32),
                    harmonic=np.tile(np.array([-1, 0], np.int32), ntraj), zs=np.full(ntraj, 100.0, np.float32))
    b.coords[1::2, 2] = 4.0
    from oracle.oracle import Lists
    L = Lists(n, b.max_long, b.max_lat, b.max_lj)     # empty static lists
    e = engine_mod.Engine(b, static_lists=L)
    e.upload_state(b.coords)
    lib = engine_mod.load()
    import torch
    out = torch.empty(ntraj * 7, dtype=torch.float64, device="cuda:0")
    rc = lib.mtg_energies_noalloc(e.h, C.c_void_p(out.data_ptr()))
    assert rc == -2
    assert b"16384" in lib.mtg_last_error_string()
    assert lib.mtg_energies_noalloc(e.h, None) == -2   # NULL output
    e.close()
