"""Python binding of the engine's C ABI (include/mtg.h) over ctypes.

``Engine`` owns one ``mtg_engine`` handle.  Every call goes through
mt_gb300/libmtg.so; there is no Python or CPU fallback: a missing library or a
failed call raises ``MtgError``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import MtgBatchTopology, MtgParams, MtgTopology, MtgTuning, ptr

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libmtg.so")

EXPORTS = {
    # name: (restype, argtypes)
    "mtg_last_error_string": (C.c_char_p, []),
    "mtg_derive_params": (C.c_int, [C.POINTER(MtgParams)]),
    "mtg_create": (C.c_int, [C.POINTER(MtgParams), C.POINTER(MtgTopology), C.POINTER(C.c_void_p)]),
    "mtg_create_batch": (C.c_int, [C.POINTER(MtgParams), C.POINTER(MtgBatchTopology), C.POINTER(C.c_void_p)]),
    "mtg_destroy": (C.c_int, [C.c_void_p]),
    "mtg_num_beads": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mtg_seed_rng": (C.c_int, [C.c_void_p, C.c_int]),
    "mtg_download_rng": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)]),
    "mtg_upload_rng": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)]),
    "mtg_generate_seeds": (C.c_int, [C.c_int, C.c_longlong, C.POINTER(C.c_uint32)]),
    "mtg_write_restart": (C.c_int, [C.c_void_p, C.c_char_p, C.c_longlong]),
    "mtg_output_open": (C.c_int, [C.c_void_p, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_int, C.c_int,
                                  C.c_int, C.c_float, C.c_char_p, C.c_char_p]),
    "mtg_output_frame": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.c_int]),
    "mtg_output_flush": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "mtg_output_close": (C.c_int, [C.c_void_p]),
    "mtg_download_flags": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_uint8), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]),
    "mtg_mt_length": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "mtg_hydrolysis_candidates": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "mtg_hydrolyse": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int8), C.POINTER(C.c_int),
                                C.POINTER(C.c_int)]),
    "mtg_hydrolysis_slots": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "mtg_count_extra": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "mtg_set_beads": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_uint8), C.c_int]),
    "mtg_read_restart": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_longlong)]),
    "mtg_upload_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "mtg_download_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "mtg_set_keep_forces": (C.c_int, [C.c_void_p, C.c_int]),
    "mtg_set_gtp": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "mtg_set_extra": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8)]),
    "mtg_set_on_tubule": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "mtg_rebuild_pairs": (C.c_int, [C.c_void_p]),
    "mtg_download_lists": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_int)] * 6),
    "mtg_list_capacity": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_int)] * 3),
    "mtg_compute_forces": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "mtg_step": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int]),
    "mtg_sync": (C.c_int, [C.c_void_p]),
    "mtg_energies": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mtg_tea_update": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "mtg_step_timed": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(C.c_float)]),
    "mtg_set_kernel_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "mtg_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.c_int]),
    "mtg_graph_kernel_launches": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.c_int]),
    "mtg_host_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    "mtg_host_free": (C.c_int, [C.c_void_p]),
    "mtg_energies_noalloc": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mtg_measure_fp32_tflops": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "mtg_device_code_version": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mtg_set_list_method": (C.c_int, [C.c_void_p, C.c_int]),
    "mtg_get_list_method": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "mtg_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(MtgTuning)]),
    "mtg_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(MtgTuning)]),
    "mtg_autotune": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(MtgTuning), C.POINTER(C.c_float)]),
    "mtg_surrogate_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "mtg_surrogate_destroy": (C.c_int, [C.c_void_p]),
    "mtg_surrogate_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "mtg_surrogate_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "mtg_surrogate_train": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int,
                                      C.c_int, C.c_float, C.c_int, C.POINTER(C.c_float)]),
    "mtg_surrogate_predict": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float)]),
    "mtg_surrogate_loss_grad": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int,
                                          C.POINTER(C.c_double), C.POINTER(C.c_float)]),
    "mtg_tea_training_data": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "mtg_set_surrogate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_float]),
    "mtg_surrogate_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "mtg_surrogate_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int]),
    "mtg_set_tea_farfield": (C.c_int, [C.c_void_p, C.c_int, C.c_float, C.c_int]),
    "mtg_tea_farfield_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_longlong)]),
    "mtg_tea_farfield_layout": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_int)] * 9),
    "mtg_tea_effective_forces": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                           C.POINTER(C.c_float)]),
}

SURROGATE_FEATURES = 32
SURROGATE_OUTPUTS = 4
SURROGATE_PARAMS = 37764

KERNEL_KINDS = ("rebuild", "step_plain", "forces", "tea_eps", "tea_beta", "tea_step", "surrogate", "recheck",
                "ff_proxies", "ff_near", "step_period", "ff_far")

_lib = None


class MtgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> C.CDLL:
    """Loads libmtg.so and declares every exported entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise MtgError(_abi.MTG_E_STATE, f"{path} is not built: run python -m mt_gb300.build")
    lib = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> int:
    if code != 0:
        raise MtgError(code, load().mtg_last_error_string().decode())
    return code


class PinnedArray:
    """numpy view of a page-locked host buffer from mtg_host_alloc."""

    def __init__(self, shape, dtype):
        self.lib = load()
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = C.c_void_p()
        check(self.lib.mtg_host_alloc(C.byref(self.ptr), n))
        buf = (C.c_char * n).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.lib.mtg_host_free(self.ptr)
            self.ptr = None


def derive_params(p: MtgParams) -> MtgParams:
    check(load().mtg_derive_params(C.byref(p)))
    return p


class Engine:
    """One batch on the GPU.  ``batch`` is a ``mt_gb300.synth.Batch``-like
    object (CSR arrays); uniform batches go through ``mtg_create`` (the
    reference layout), ragged ones through ``mtg_create_batch``."""

    def __init__(self, batch, static_lists=None, force_ragged: bool = False):
        self.lib = load()
        self.batch = batch
        self.params = batch.params
        self._keep = []
        h = C.c_void_p()
        if batch.uniform_ntot and not force_ragged and static_lists is None:
            n = batch.uniform_ntot
            t = MtgTopology()
            t.Ntot, t.Ntr = n, batch.ntraj
            t.maxHarmonicPerMonomer = batch.max_h
            hc = np.ascontiguousarray(batch.harmonic_count[:n])
            hh = np.ascontiguousarray(batch.harmonic[:batch.max_h * n])
            fx = np.ascontiguousarray(batch.fixed[:n])
            mt = np.ascontiguousarray(batch.mon_type[:n])
            self._keep += [hc, hh, fx, mt]
            t.harmonicCount, t.harmonic = ptr(hc, C.c_int), ptr(hh, C.c_int)
            t.maxLongitudinalPerMonomer, t.maxLateralPerMonomer = batch.max_long, batch.max_lat
            t.maxLJPerMonomer = batch.max_lj
            t.fixed, t.mon_type = ptr(fx, C.c_uint8), ptr(mt, C.c_int)
            t.extra, t.gtp = ptr(batch.extra, C.c_uint8), ptr(batch.gtp, C.c_int)
            t.on_tubule_cur, t.zs = ptr(batch.on_tubule, C.c_int), ptr(batch.zs, C.c_float)
            check(self.lib.mtg_create(C.byref(batch.params), C.byref(t), C.byref(h)))
        else:
            t = MtgBatchTopology()
            t.ntraj = batch.ntraj
            t.offsets = ptr(batch.offsets, C.c_int)
            t.maxHarmonicPerMonomer = batch.max_h
            t.harmonicCount, t.harmonic = ptr(batch.harmonic_count, C.c_int), ptr(batch.harmonic, C.c_int)
            t.maxLongitudinalPerMonomer, t.maxLateralPerMonomer = batch.max_long, batch.max_lat
            t.maxLJPerMonomer = batch.max_lj
            if static_lists is not None:
                L = static_lists
                self._keep += [L.long_count, L.lon, L.lat_count, L.lat]
                t.longitudinalCount, t.longitudinal = ptr(L.long_count, C.c_int), ptr(L.lon, C.c_int)
                t.lateralCount, t.lateral = ptr(L.lat_count, C.c_int), ptr(L.lat, C.c_int)
            t.fixed, t.extra = ptr(batch.fixed, C.c_uint8), ptr(batch.extra, C.c_uint8)
            t.mon_type, t.gtp = ptr(batch.mon_type, C.c_int), ptr(batch.gtp, C.c_int)
            t.on_tubule_cur, t.zs = ptr(batch.on_tubule, C.c_int), ptr(batch.zs, C.c_float)
            check(self.lib.mtg_create_batch(C.byref(batch.params), C.byref(t), C.byref(h)))
        self.h = h
        nb, nt = C.c_int(), C.c_int()
        check(self.lib.mtg_num_beads(self.h, C.byref(nb), C.byref(nt)))
        self.nb, self.nt = nb.value, nt.value

    # ------------------------------------------------------------ lifecycle
    def close(self):
        if getattr(self, "h", None):
            self.lib.mtg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ----------------------------------------------------------------- state
    def upload_state(self, coords: np.ndarray):
        c = np.ascontiguousarray(coords, np.float32)
        assert c.shape == (self.nb, 7)
        check(self.lib.mtg_upload_state(self.h, ptr(c, C.c_float)))

    def download_state(self, forces: bool = False):
        r = np.zeros((self.nb, 7), np.float32)
        f = np.zeros((self.nb, 7), np.float32) if forces else None
        check(self.lib.mtg_download_state(self.h, ptr(r, C.c_float), ptr(f, C.c_float)))
        return (r, f) if forces else r

    def set_keep_forces(self, keep: bool = True):
        check(self.lib.mtg_set_keep_forces(self.h, int(keep)))

    def seed_rng(self, seed: int):
        check(self.lib.mtg_seed_rng(self.h, seed))

    def download_rng(self) -> np.ndarray:
        s = np.zeros(8 * self.nb, np.uint32)
        check(self.lib.mtg_download_rng(self.h, ptr(s, C.c_uint32)))
        return s

    def upload_rng(self, seeds: np.ndarray):
        s = np.ascontiguousarray(seeds, np.uint32)
        assert s.size == 8 * self.nb
        check(self.lib.mtg_upload_rng(self.h, ptr(s, C.c_uint32)))

    def write_restart(self, path: str, step: int):
        check(self.lib.mtg_write_restart(self.h, os.fsencode(path), step))

    def read_restart(self, path: str) -> int:
        """Loads the restart file; returns the step to resume from."""
        st = C.c_longlong()
        check(self.lib.mtg_read_restart(self.h, os.fsencode(path), C.byref(st)))
        return st.value

    def output_open(self, xyz_paths, ang_paths, nfile: int, npriv: int, nsavc: int, delta: float,
                    remark2: str | None = None, energy_path: str | None = None):
        """DCD files of every trajectory (coordinates, angles); see mtg_output_open."""
        xa = (C.c_char_p * self.nt)(*[os.fsencode(p) for p in xyz_paths])
        aa = (C.c_char_p * self.nt)(*[os.fsencode(p) for p in ang_paths])
        check(self.lib.mtg_output_open(self.h, xa, aa, nfile, npriv, nsavc, delta,
                                       None if remark2 is None else remark2.encode(),
                                       None if energy_path is None else os.fsencode(energy_path)))

    def output_frame(self, step: int, frame: bool = True, energies: bool = False):
        check(self.lib.mtg_output_frame(self.h, step, int(frame), int(energies)))

    def output_flush(self) -> int:
        n = C.c_longlong()
        check(self.lib.mtg_output_flush(self.h, C.byref(n)))
        return n.value

    def output_close(self):
        check(self.lib.mtg_output_close(self.h))

    def download_flags(self):
        """(gtp, extra, on_tubule_cur, on_tubule_prev) per bead."""
        g = np.zeros(self.nb, np.int32)
        x = np.zeros(self.nb, np.uint8)
        c = np.zeros(self.nb, np.int32)
        p = np.zeros(self.nb, np.int32)
        check(self.lib.mtg_download_flags(self.h, ptr(g, C.c_int), ptr(x, C.c_uint8), ptr(c, C.c_int),
                                          ptr(p, C.c_int)))
        return g, x, c, p

    def mt_length(self, save_prev: bool):
        out = np.zeros(self.nt, np.int32)
        check(self.lib.mtg_mt_length(self.h, int(save_prev), ptr(out, C.c_int)))
        return out

    def hydrolysis_candidates(self) -> int:
        n = C.c_int()
        check(self.lib.mtg_hydrolysis_candidates(self.h, C.byref(n)))
        return n.value

    def hydrolyse(self, prob, events: bool = False):
        """Applies hydrolysis with one number per candidate; returns
        (n_hydrolysed, n_restored, events [max_dimers, ntraj] or None)."""
        p = np.ascontiguousarray(prob, np.float64)
        md = C.c_int()
        check(self.lib.mtg_hydrolysis_slots(self.h, C.byref(md)))
        ev = np.zeros((md.value, self.nt), np.int8) if events else None
        nh, nr = C.c_int(), C.c_int()
        check(self.lib.mtg_hydrolyse(self.h, ptr(p, C.c_double), len(p), ptr(ev, C.c_int8), C.byref(nh),
                                     C.byref(nr)))
        return nh.value, nr.value, ev

    def count_extra(self):
        out = np.zeros(self.nt, np.int32)
        check(self.lib.mtg_count_extra(self.h, ptr(out, C.c_int)))
        return out

    def set_beads(self, idx, coords, extra=None):
        i = np.ascontiguousarray(idx, np.int32)
        c = np.ascontiguousarray(coords, np.float32).reshape(len(i), 7)
        x = None if extra is None else np.ascontiguousarray(extra, np.uint8)
        check(self.lib.mtg_set_beads(self.h, ptr(i, C.c_int), ptr(c, C.c_float), ptr(x, C.c_uint8), len(i)))

    def set_gtp(self, gtp):
        a = np.ascontiguousarray(gtp, np.int32)
        check(self.lib.mtg_set_gtp(self.h, ptr(a, C.c_int)))

    def set_extra(self, extra):
        a = np.ascontiguousarray(extra, np.uint8)
        check(self.lib.mtg_set_extra(self.h, ptr(a, C.c_uint8)))

    def set_on_tubule(self, on):
        a = np.ascontiguousarray(on, np.int32)
        check(self.lib.mtg_set_on_tubule(self.h, ptr(a, C.c_int)))

    # ---------------------------------------------------------------- compute
    def rebuild_pairs(self):
        check(self.lib.mtg_rebuild_pairs(self.h))

    def set_list_method(self, method: int):
        """0 auto, 1 brute-force tiles, 2 cell list."""
        check(self.lib.mtg_set_list_method(self.h, method))

    def list_method(self) -> int:
        m = C.c_int()
        check(self.lib.mtg_get_list_method(self.h, C.byref(m)))
        return m.value

    def lists(self):
        """(counts, entries) per kind in the reference layout (bead-major, cap per bead)."""
        ml, mt, mj = C.c_int(), C.c_int(), C.c_int()
        check(self.lib.mtg_list_capacity(self.h, C.byref(ml), C.byref(mt), C.byref(mj)))
        out = {}
        a = [np.zeros(self.nb, np.int32), np.zeros(self.nb * mj.value, np.int32),
             np.zeros(self.nb, np.int32), np.zeros(self.nb * ml.value, np.int32),
             np.zeros(self.nb, np.int32), np.zeros(self.nb * mt.value, np.int32)]
        check(self.lib.mtg_download_lists(self.h, *[ptr(x, C.c_int) for x in a]))
        out["lj"] = (a[0], a[1], mj.value)
        out["long"] = (a[2], a[3], ml.value)
        out["lat"] = (a[4], a[5], mt.value)
        return out

    def list_of_lists(self, kind: str):
        cnt, arr, cap = self.lists()[kind]
        return [arr[cap * i: cap * i + cnt[i]].tolist() for i in range(self.nb)]

    def compute_forces(self) -> np.ndarray:
        f = np.zeros((self.nb, 7), np.float32)
        check(self.lib.mtg_compute_forces(self.h, ptr(f, C.c_float)))
        return f

    def step(self, first_step: int, nsteps: int):
        check(self.lib.mtg_step(self.h, C.c_longlong(first_step), C.c_int(nsteps)))

    def step_raw(self, first_step: int, nsteps: int) -> int:
        """mtg_step returning its status instead of raising."""
        return self.lib.mtg_step(self.h, C.c_longlong(first_step), C.c_int(nsteps))

    def step_timed(self, first_step: int, nsteps: int) -> float:
        """mtg_step between two CUDA events on the engine's stream; returns device ms."""
        ms = C.c_float()
        check(self.lib.mtg_step_timed(self.h, C.c_longlong(first_step), C.c_int(nsteps), C.byref(ms)))
        return ms.value

    def set_kernel_timing(self, on: bool = True):
        check(self.lib.mtg_set_kernel_timing(self.h, int(on)))

    def kernel_times(self, reset: bool = False):
        """{kind: (total_ms, launches)} of the timed kernel launches."""
        t = (C.c_double * len(KERNEL_KINDS))()
        n = (C.c_longlong * len(KERNEL_KINDS))()
        check(self.lib.mtg_kernel_times(self.h, t, n, int(reset)))
        return {k: (t[i], n[i]) for i, k in enumerate(KERNEL_KINDS)}

    def graph_kernel_launches(self, reset: bool = False) -> int:
        """Kernel nodes replayed from the step graphs since the last reset."""
        n = C.c_longlong(0)
        check(self.lib.mtg_graph_kernel_launches(self.h, C.byref(n), int(reset)))
        return n.value

    def tuning(self) -> dict:
        t = MtgTuning()
        check(self.lib.mtg_get_tuning(self.h, C.byref(t)))
        return {"list_method": t.list_method, "step_block": t.step_block, "tea_slices": t.tea_slices,
                "tea_jparts": t.tea_jparts, "plain_persistent": t.plain_persistent}

    def set_tuning(self, list_method: int, step_block: int, tea_slices: int, tea_jparts: int = 1,
                   plain_persistent: int = 0):
        t = MtgTuning(list_method, step_block, tea_slices, tea_jparts, plain_persistent)
        check(self.lib.mtg_set_tuning(self.h, C.byref(t)))

    def autotune(self, first_step: int, trial_steps: int, cache: str | None = None, key: str | None = None):
        """Runs mtg_autotune, or applies a cached result for `key` (the GPU name
        and the workload signature) from the JSON file `cache`."""
        import json
        if cache and key and os.path.exists(cache):
            try:
                entry = json.load(open(cache)).get(key)
            except (OSError, ValueError):
                entry = None
            if entry:
                self.set_tuning(**entry["tuning"])
                return dict(entry, cached=True)
        t = MtgTuning()
        ms = C.c_float()
        check(self.lib.mtg_autotune(self.h, C.c_longlong(first_step), trial_steps, C.byref(t), C.byref(ms)))
        entry = {"tuning": {"list_method": t.list_method, "step_block": t.step_block, "tea_slices": t.tea_slices,
                            "tea_jparts": t.tea_jparts, "plain_persistent": t.plain_persistent},
                 "trial_ms": ms.value, "cached": False}
        if cache and key:
            try:
                data = json.load(open(cache)) if os.path.exists(cache) else {}
            except (OSError, ValueError):
                data = {}
            data[key] = {k: v for k, v in entry.items() if k != "cached"}
            os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
            json.dump(data, open(cache, "w"), indent=1)
        return entry

    def tea_training_data(self, targets: bool = True):
        """(descriptors [nb, 32], targets [nb, 4] = C_i, beta) of the current state."""
        X = np.zeros((self.nb, SURROGATE_FEATURES), np.float32)
        T = np.zeros((self.nb, SURROGATE_OUTPUTS), np.float32) if targets else None
        check(self.lib.mtg_tea_training_data(self.h, ptr(X, C.c_float), ptr(T, C.c_float)))
        return X, T

    def set_surrogate(self, surrogate, recheck_every: int = 100, max_err: float = 0.01):
        check(self.lib.mtg_set_surrogate(self.h, surrogate.h if surrogate else None, recheck_every, max_err))
        self._surrogate = surrogate

    def surrogate_status(self):
        fb, nr, err = C.c_int(), C.c_int(), C.c_double()
        check(self.lib.mtg_surrogate_status(self.h, C.byref(fb), C.byref(nr), C.byref(err)))
        return {"fell_back": bool(fb.value), "rechecks": nr.value, "last_error": err.value}

    def set_tea_farfield(self, on: bool = True, theta: float = 0.85, refresh_every: int = 0):
        check(self.lib.mtg_set_tea_farfield(self.h, int(on), theta, refresh_every))

    def tea_farfield_stats(self):
        nl, npairs, ppairs = C.c_int(), C.c_longlong(), C.c_longlong()
        check(self.lib.mtg_tea_farfield_stats(self.h, C.byref(nl), C.byref(npairs), C.byref(ppairs)))
        return {"leaves": nl.value, "near_pairs": npairs.value, "proxy_pairs": ppairs.value}

    def tea_farfield_layout(self):
        """(leaf_start, leaf_bead, near_start, near, node_range, node_parent, far_start, far) of the tree
        (nodes 0 .. nleaf-1 are the leaves)."""
        sz = np.zeros(5, np.int32)
        nul = C.cast(None, C.POINTER(C.c_int))
        check(self.lib.mtg_tea_farfield_layout(self.h, ptr(sz, C.c_int), *([nul] * 8)))
        nl, nbl, nnear, nn, nfar = (int(v) for v in sz)
        a = [np.zeros(nl + 1, np.int32), np.zeros(max(nbl, 1), np.int32), np.zeros(nl + 1, np.int32),
             np.zeros(max(nnear, 1), np.int32), np.zeros(max(2 * nn, 1), np.int32), np.zeros(max(nn, 1), np.int32),
             np.zeros(nn + 1, np.int32), np.zeros(max(nfar, 1), np.int32)]
        check(self.lib.mtg_tea_farfield_layout(self.h, ptr(sz, C.c_int), *[ptr(x, C.c_int) for x in a]))
        return (a[0], a[1][:nbl], a[2], a[3][:nnear], a[4][:2 * nn], a[5][:nn], a[6], a[7][:nfar])

    def tea_effective_forces(self, exact: bool = True, farfield: bool = True):
        """(feff_exact, feff_ff, rforce) [nb, 4] of the current state from one draw of random forces."""
        fe = np.zeros((self.nb, 4), np.float32) if exact else None
        ff = np.zeros((self.nb, 4), np.float32) if farfield else None
        rf = np.zeros((self.nb, 4), np.float32)
        check(self.lib.mtg_tea_effective_forces(self.h, ptr(fe, C.c_float), ptr(ff, C.c_float), ptr(rf, C.c_float)))
        return fe, ff, rf

    def energies(self, per_bead: bool = False):
        pt = np.zeros((self.nt, 7), np.float64)
        pb = np.zeros((self.nb, 7), np.float64) if per_bead else None
        check(self.lib.mtg_energies(self.h, ptr(pb, C.c_double), ptr(pt, C.c_double)))
        return (pt, pb) if per_bead else pt

    def tea_update(self):
        eps = np.zeros(self.nt, np.float64)
        beta = np.zeros(self.nt, np.float32)
        ci = np.zeros((self.nb, 4), np.float32)
        rc = self.lib.mtg_tea_update(self.h, ptr(eps, C.c_double), ptr(beta, C.c_float), ptr(ci, C.c_float))
        return eps, beta, ci, rc


class Surrogate:
    """The learned-TEA network (mtg_surrogate_*)."""

    def __init__(self, device: int = 0, seed: int = 1):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.mtg_surrogate_create(device, seed, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.mtg_surrogate_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.zeros(SURROGATE_PARAMS, np.float32)
        n = np.zeros(72, np.float32)
        check(self.lib.mtg_surrogate_get_params(self.h, ptr(p, C.c_float), ptr(n, C.c_float)))
        return p, n

    def set_params(self, params=None, norm=None):
        pp = None if params is None else np.ascontiguousarray(params, np.float32)
        nn = None if norm is None else np.ascontiguousarray(norm, np.float32)
        check(self.lib.mtg_surrogate_set_params(self.h, ptr(pp, C.c_float), ptr(nn, C.c_float)))

    def train(self, X, T, epochs: int = 20, batch: int = 4096, lr: float = 1e-3, seed: int = 0):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        losses = np.zeros(epochs, np.float32)
        check(self.lib.mtg_surrogate_train(self.h, ptr(X, C.c_float), ptr(T, C.c_float), len(X), epochs, batch,
                                           lr, seed, ptr(losses, C.c_float)))
        return losses

    def set_wait_limit(self, polls: int = -1):
        """Polls of the inference's bounded waits for the tensor cores (< 0: default)."""
        check(self.lib.mtg_surrogate_set_wait_limit(self.h, polls))

    def predict_raw(self, X):
        """mtg_surrogate_predict returning (status, Y) instead of raising."""
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((len(X), SURROGATE_OUTPUTS), np.float32)
        rc = self.lib.mtg_surrogate_predict(self.h, ptr(X, C.c_float), len(X), ptr(Y, C.c_float))
        return rc, Y

    def predict(self, X):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((len(X), SURROGATE_OUTPUTS), np.float32)
        check(self.lib.mtg_surrogate_predict(self.h, ptr(X, C.c_float), len(X), ptr(Y, C.c_float)))
        return Y

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        g = np.zeros(SURROGATE_PARAMS, np.float32)
        loss = C.c_double()
        check(self.lib.mtg_surrogate_loss_grad(self.h, ptr(X, C.c_float), ptr(T, C.c_float), len(X), C.byref(loss),
                                               ptr(g, C.c_float)))
        return loss.value, g


def generate_seeds(rseed: int, nstreams: int) -> np.ndarray:
    """HybridTaus states of nstreams streams from rseed (mtg_generate_seeds)."""
    out = np.zeros(4 * nstreams, np.uint32)
    check(load().mtg_generate_seeds(rseed, nstreams, ptr(out, C.c_uint32)))
    return out


def split_by_beads(offsets, nparts: int):
    """Contiguous groups of trajectories with about equal bead counts: part k
    ends at the first trajectory boundary at or past k/nparts of the beads.
    Returns [(t0, t1)] covering every trajectory once (parts may be empty
    when there are fewer trajectories than parts)."""
    offsets = np.asarray(offsets, np.int64)
    nt, nb = len(offsets) - 1, int(offsets[-1])
    if nparts < 1:
        raise ValueError("nparts must be positive")
    cuts = [0]
    for k in range(1, nparts):
        t = int(np.searchsorted(offsets, k * nb / nparts, side="left"))
        cuts.append(min(max(t, cuts[-1]), nt))
    cuts.append(nt)
    return [(cuts[k], cuts[k + 1]) for k in range(nparts)]


class ShardedEngine:
    """One batch over several GPUs, the replacement of the reference's MPI
    replicas (src/main.cpp:27-48): trajectories never interact, so the batch
    is cut into contiguous groups of about equal bead counts
    (split_by_beads), each group runs on its own engine, device and stream,
    and calls fan out to the engines (concurrently, one host thread each) and
    gather their results in batch order.  No collective and no peer access.
    The noise streams are the ones an engine of the whole batch would draw
    (mtg_generate_seeds of the whole batch, sliced per group), so the result
    equals that engine's bit for bit."""

    def __init__(self, batch, devices):
        import concurrent.futures as cf

        from . import synth
        self.batch = batch
        parts = split_by_beads(batch.offsets, len(devices))
        self.parts = [(t0, t1, d) for (t0, t1), d in zip(parts, devices) if t1 > t0]
        self.nb, self.nt = batch.nbeads, batch.ntraj
        self.engines = []
        for t0, t1, d in self.parts:
            sub = synth.sub_batch(batch, t0, t1)
            sub.params.device = d
            self.engines.append(Engine(sub))
        self.ranges = [(int(batch.offsets[t0]), int(batch.offsets[t1])) for t0, t1, _ in self.parts]
        seeds = generate_seeds(int(batch.params.rseed), 2 * self.nb).reshape(2, self.nb, 4)
        for e, (b0, b1) in zip(self.engines, self.ranges):
            e.upload_rng(np.ascontiguousarray(seeds[:, b0:b1]).reshape(-1))
        self._pool = cf.ThreadPoolExecutor(max_workers=len(self.engines))

    def _each(self, fn):
        return list(self._pool.map(fn, range(len(self.engines))))

    def upload_state(self, coords):
        c = np.ascontiguousarray(coords, np.float32)
        self._each(lambda k: self.engines[k].upload_state(c[self.ranges[k][0]:self.ranges[k][1]]))

    def download_state(self):
        return np.concatenate(self._each(lambda k: self.engines[k].download_state()))

    def download_rng(self):
        parts = self._each(lambda k: self.engines[k].download_rng().reshape(2, -1, 4))
        return np.concatenate(parts, axis=1).reshape(-1)

    def step(self, first_step: int, nsteps: int):
        self._each(lambda k: self.engines[k].step(first_step, nsteps))

    def energies(self):
        return np.concatenate(self._each(lambda k: self.engines[k].energies()))

    def close(self):
        for e in self.engines:
            e.close()
        self.engines = []
        self._pool.shutdown()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
