"""Python driver of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/liboracle.so (the C restatement, ``kind="orc"``) or
oracle/_ref/libmtref.so (the reference's own kernel bodies compiled as host
code, ``kind="ref"``, FP32 only) and runs them on ``mt_gb300.synth.Batch``
objects.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
import this module.

Batches are processed in the reference's uniform layout; a ragged batch is
run one trajectory at a time (Ntr = 1 each), which is how the reference would
have to run it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from mt_gb300._abi import MtgTopology, ptr

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmtref.so")

_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)


def build(ref: bool = False) -> None:
    """Compiles the oracle (and, with ref=True, the reference harness)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


class _Views:
    """Keeps the numpy arrays behind an MtgTopology alive."""

    def __init__(self, batch, t0: int, t1: int):
        off = batch.offsets
        b0, b1 = int(off[t0]), int(off[t1])
        ntot = int(off[t0 + 1] - off[t0])
        ntr = t1 - t0
        if any(int(off[t + 1] - off[t]) != ntot for t in range(t0, t1)):
            raise ValueError("trajectories of one oracle call must have equal sizes")
        h = batch.max_h
        self.ntot, self.ntr, self.b0, self.b1 = ntot, ntr, b0, b1
        self.harmonic_count = np.ascontiguousarray(batch.harmonic_count[b0:b0 + ntot])
        self.harmonic = np.ascontiguousarray(batch.harmonic[h * b0:h * (b0 + ntot)])
        self.fixed = np.ascontiguousarray(batch.fixed[b0:b0 + ntot])
        self.mon_type = np.ascontiguousarray(batch.mon_type[b0:b0 + ntot])
        self.extra = np.ascontiguousarray(batch.extra[b0:b1])
        self.gtp = np.ascontiguousarray(batch.gtp[b0:b1])
        self.on_tubule = np.ascontiguousarray(batch.on_tubule[b0:b1])
        self.zs = np.ascontiguousarray(batch.zs[t0:t1])
        t = MtgTopology()
        t.Ntot, t.Ntr = ntot, ntr
        t.maxHarmonicPerMonomer = h
        t.harmonicCount = ptr(self.harmonic_count, C.c_int)
        t.harmonic = ptr(self.harmonic, C.c_int)
        t.maxLongitudinalPerMonomer = batch.max_long
        t.maxLateralPerMonomer = batch.max_lat
        t.maxLJPerMonomer = batch.max_lj
        t.fixed = ptr(self.fixed, C.c_uint8)
        t.mon_type = ptr(self.mon_type, C.c_int)
        t.extra = ptr(self.extra, C.c_uint8)
        t.gtp = ptr(self.gtp, C.c_int)
        t.on_tubule_cur = ptr(self.on_tubule, C.c_int)
        t.zs = ptr(self.zs, C.c_float)
        self.top = t


class Lists:
    """Neighbour lists in the reference layout for beads b0..b1 of a batch."""

    def __init__(self, n: int, max_long: int, max_lat: int, max_lj: int):
        self.max_long, self.max_lat, self.max_lj = max_long, max_lat, max_lj
        self.long_count = np.zeros(n, np.int32)
        self.lon = np.zeros(n * max_long, np.int32)
        self.lat_count = np.zeros(n, np.int32)
        self.lat = np.zeros(n * max_lat, np.int32)
        self.lj_count = np.zeros(n, np.int32)
        self.lj = np.zeros(n * max_lj, np.int32)

    def as_lists(self, kind: str):
        cnt, arr, cap = {"lj": (self.lj_count, self.lj, self.max_lj),
                         "long": (self.long_count, self.lon, self.max_long),
                         "lat": (self.lat_count, self.lat, self.max_lat)}[kind]
        return [arr[cap * i: cap * i + cnt[i]].tolist() for i in range(len(cnt))]


class Oracle:
    """One loaded oracle library at one precision."""

    def __init__(self, kind: str = "orc", precision: str = "f32"):
        path = ORACLE_SO if kind == "orc" else REF_SO
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} not built")
        if kind == "ref" and precision != "f32":
            raise ValueError("the reference harness is FP32 only")
        self.lib = C.CDLL(path)
        self.kind = kind
        self.prec = precision
        self.dtype = np.float32 if precision == "f32" else np.float64
        self.rp = _f32p if precision == "f32" else _f64p
        self.pre = "orc_" if kind == "orc" else "ref_"

    def _fn(self, name: str, suffixed: bool = True):
        return getattr(self.lib, self.pre + name + ("_" + self.prec if suffixed else ""))

    # ------------------------------------------------------------- RNG
    def generate_seeds(self, seed: int, nstreams: int) -> np.ndarray:
        out = np.zeros(4 * nstreams, np.uint32)
        self._fn("generate_seeds", False)(C.c_int(seed), C.c_int(nstreams), ptr(out, C.c_uint32))
        return out

    def rforce(self, state: np.ndarray, n: int) -> np.ndarray:
        """n rforce() draws on one stream; state (4 uint32) is advanced in place."""
        out = np.zeros(4 * n, self.dtype)
        self._fn("rforce")(ptr(state, C.c_uint32), C.c_int(n), out.ctypes.data_as(self.rp))
        return out.reshape(n, 4)

    # ---------------------------------------------------- per-call helpers
    def _coords(self, coords: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(coords, dtype=self.dtype)

    def _trajectory_groups(self, batch):
        """Runs of trajectories that can share one uniform oracle call."""
        if batch.uniform_ntot:
            return [(0, batch.ntraj)]
        return [(t, t + 1) for t in range(batch.ntraj)]

    def lists(self, batch, coords: np.ndarray, lj: bool = True, pairs: bool = True):
        """LJ list (LJ_kernel) and assembly lists (pairs_kernel) of all beads."""
        L = Lists(batch.nbeads, batch.max_long, batch.max_lat, batch.max_lj)
        ovf = C.c_int(0)
        x = self._coords(coords)
        for t0, t1 in self._trajectory_groups(batch):
            v = _Views(batch, t0, t1)
            b0, b1 = v.b0, v.b1
            xs = np.ascontiguousarray(x[b0:b1])
            n = b1 - b0
            if lj:
                cnt = np.zeros(n, np.int32)
                arr = np.zeros(n * batch.max_lj, np.int32)
                self._fn("lj_list")(C.byref(batch.params), C.byref(v.top), xs.ctypes.data_as(self.rp),
                                    C.c_int(batch.max_lj), ptr(cnt, C.c_int), ptr(arr, C.c_int), C.byref(ovf))
                L.lj_count[b0:b1] = cnt
                L.lj[batch.max_lj * b0:batch.max_lj * b1] = arr
            if pairs:
                lc = np.zeros(n, np.int32)
                la = np.zeros(n * batch.max_long, np.int32)
                tc = np.zeros(n, np.int32)
                ta = np.zeros(n * batch.max_lat, np.int32)
                self._fn("pairs_list")(C.byref(batch.params), C.byref(v.top), xs.ctypes.data_as(self.rp),
                                       C.c_int(batch.max_long), ptr(lc, C.c_int), ptr(la, C.c_int),
                                       C.c_int(batch.max_lat), ptr(tc, C.c_int), ptr(ta, C.c_int), C.byref(ovf))
                L.long_count[b0:b1] = lc
                L.lon[batch.max_long * b0:batch.max_long * b1] = la
                L.lat_count[b0:b1] = tc
                L.lat[batch.max_lat * b0:batch.max_lat * b1] = ta
        L.overflow = bool(ovf.value)
        return L

    def _list_args(self, L: Lists, batch, b0: int, b1: int):
        sl = lambda a, cap: np.ascontiguousarray(a[cap * b0:cap * b1])
        keep = [np.ascontiguousarray(L.long_count[b0:b1]), sl(L.lon, L.max_long),
                np.ascontiguousarray(L.lat_count[b0:b1]), sl(L.lat, L.max_lat),
                np.ascontiguousarray(L.lj_count[b0:b1]), sl(L.lj, L.max_lj)]
        args = [C.c_int(L.max_long), ptr(keep[0], C.c_int), ptr(keep[1], C.c_int),
                C.c_int(L.max_lat), ptr(keep[2], C.c_int), ptr(keep[3], C.c_int),
                C.c_int(L.max_lj), ptr(keep[4], C.c_int), ptr(keep[5], C.c_int)]
        return keep, args

    def forces(self, batch, coords: np.ndarray, L: Lists) -> np.ndarray:
        """compute_kernel forces, Coord AoS [nbeads, 7] (zero for extra beads)."""
        x = self._coords(coords)
        f = np.zeros_like(x)
        for t0, t1 in self._trajectory_groups(batch):
            v = _Views(batch, t0, t1)
            keep, args = self._list_args(L, batch, v.b0, v.b1)
            xs = np.ascontiguousarray(x[v.b0:v.b1])
            fs = np.zeros_like(xs)
            self._fn("forces")(C.byref(batch.params), C.byref(v.top), xs.ctypes.data_as(self.rp), *args,
                               fs.ctypes.data_as(self.rp))
            f[v.b0:v.b1] = fs
        return f

    def energies(self, batch, coords: np.ndarray, L: Lists) -> np.ndarray:
        """energy_kernel per-bead terms [nbeads, 7] (double)."""
        x = self._coords(coords)
        en = np.zeros((batch.nbeads, 7), np.float64)
        for t0, t1 in self._trajectory_groups(batch):
            v = _Views(batch, t0, t1)
            keep, args = self._list_args(L, batch, v.b0, v.b1)
            xs = np.ascontiguousarray(x[v.b0:v.b1])
            es = np.zeros((v.b1 - v.b0, 7), np.float64)
            self._fn("energies")(C.byref(batch.params), C.byref(v.top), xs.ctypes.data_as(self.rp), *args,
                                 ptr(es, C.c_double))
            en[v.b0:v.b1] = es
        return en

    def run(self, batch, coords: np.ndarray, seeds: np.ndarray, first_step: int, nsteps: int,
            L: Lists | None = None, tea_ci=None, tea_beta=None):
        """Step loop of compute() without I/O; returns (coords, forces, seeds, lists, status, tea_ci, tea_beta).

        seeds: [8*nbeads] uint32 in the engine's order (stream g = xyz noise of
        bead g, stream g + nbeads = its angle noise)."""
        x = self._coords(coords).copy()
        f = np.zeros_like(x)
        nb = batch.nbeads
        s_all = seeds.copy()
        L = L or Lists(nb, batch.max_long, batch.max_lat, batch.max_lj)
        ci = np.zeros((nb, 4), self.dtype) if tea_ci is None else np.ascontiguousarray(tea_ci, self.dtype).copy()
        beta = np.zeros(batch.ntraj, self.dtype) if tea_beta is None else \
            np.ascontiguousarray(tea_beta, self.dtype).copy()
        status = 0
        for t0, t1 in self._trajectory_groups(batch):
            v = _Views(batch, t0, t1)
            b0, b1 = v.b0, v.b1
            n = b1 - b0
            xs = np.ascontiguousarray(x[b0:b1])
            fs = np.zeros_like(xs)
            # the reference's stream p / p + Ntot*Ntr for the sub-batch
            ss = np.concatenate([s_all[4 * b0:4 * b1], s_all[4 * (nb + b0):4 * (nb + b1)]]).copy()
            keep, _ = self._list_args(L, batch, b0, b1)
            cis = np.ascontiguousarray(ci[b0:b1])
            bs = np.ascontiguousarray(beta[t0:t1])
            st = self._fn("run")(C.byref(batch.params), C.byref(v.top), xs.ctypes.data_as(self.rp),
                                 fs.ctypes.data_as(self.rp), ptr(ss, C.c_uint32),
                                 C.c_int(L.max_long), ptr(keep[0], C.c_int), ptr(keep[1], C.c_int),
                                 C.c_int(L.max_lat), ptr(keep[2], C.c_int), ptr(keep[3], C.c_int),
                                 C.c_int(L.max_lj), ptr(keep[4], C.c_int), ptr(keep[5], C.c_int),
                                 C.c_longlong(first_step), C.c_int(nsteps),
                                 cis.ctypes.data_as(self.rp), bs.ctypes.data_as(self.rp))
            status = status or st
            x[b0:b1] = xs
            f[b0:b1] = fs
            s_all[4 * b0:4 * b1] = ss[:4 * n]
            s_all[4 * (nb + b0):4 * (nb + b1)] = ss[4 * n:]
            L.long_count[b0:b1] = keep[0]
            L.lon[L.max_long * b0:L.max_long * b1] = keep[1]
            L.lat_count[b0:b1] = keep[2]
            L.lat[L.max_lat * b0:L.max_lat * b1] = keep[3]
            L.lj_count[b0:b1] = keep[4]
            L.lj[L.max_lj * b0:L.max_lj * b1] = keep[5]
            ci[b0:b1] = cis
            beta[t0:t1] = bs
        return x, f, s_all, L, status, ci, beta

    # ---------------------------------------------------------------- TEA
    def tea_epsilon(self, batch, coords: np.ndarray):
        x = self._coords(coords)
        ci = np.zeros((batch.nbeads, 4), self.dtype)
        eps = np.zeros(batch.nbeads, self.dtype)
        for t0, t1 in self._trajectory_groups(batch):
            v = _Views(batch, t0, t1)
            xs = np.ascontiguousarray(x[v.b0:v.b1])
            cs = np.zeros((v.b1 - v.b0, 4), self.dtype)
            es = np.zeros(v.b1 - v.b0, self.dtype)
            self._fn("tea_epsilon")(C.byref(batch.params), C.byref(v.top), xs.ctypes.data_as(self.rp),
                                    cs.ctypes.data_as(self.rp), es.ctypes.data_as(self.rp))
            ci[v.b0:v.b1] = cs
            eps[v.b0:v.b1] = es
        return ci, eps

    def tea_beta(self, batch, eps: np.ndarray):
        """updateTea's FP64 reduction (restated in both oracle libraries: use the C oracle)."""
        lib = C.CDLL(ORACLE_SO)
        fn = getattr(lib, "orc_tea_beta_" + self.prec)
        eps_t = np.zeros(batch.ntraj, np.float64)
        beta = np.zeros(batch.ntraj, self.dtype)
        status = 0
        for t0, t1 in self._trajectory_groups(batch):
            v = _Views(batch, t0, t1)
            es = np.ascontiguousarray(eps[v.b0:v.b1], self.dtype)
            et = np.zeros(t1 - t0, np.float64)
            bt = np.zeros(t1 - t0, self.dtype)
            status = fn(C.byref(batch.params), C.byref(v.top), es.ctypes.data_as(self.rp), ptr(et, C.c_double),
                        bt.ctypes.data_as(self.rp)) or status
            eps_t[t0:t1] = et
            beta[t0:t1] = bt
        return eps_t, beta, status
