"""Benchmark of the Brownian/Langevin hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl mtg|reference]

The default workload is the headline comparison: exact TEA against learned
TEA (the surrogate network in the step loop, re-checked by exact TEA every
100 steps, fallback above 1% RMS mobility error) on 64 trajectories of
13 PF x 200 monomers + 3000 free monomers; `value` is the learned path's
monomer-steps/s (the exact path's if the learned one fell back), and the
line carries both.  One bench step = one re-check period (100 MD steps)
there, and one pair-list period (``ljpairsupdatefreq`` = 10 MD steps: one
list rebuild + 10 force/update steps) for the other workloads.  The metric
is monomer-steps/s = active (non-extra) beads x MD steps / seconds.

value     device time of the K timed bench steps (CUDA events on the engine's
          stream), inputs resident in HBM; L2 is flushed (256 MB write)
          before every timed bench step, outside the timed interval.
e2e       the same steps through the C ABI with host buffers: every step
          uploads the state from pinned host memory, runs, and downloads the
          state (wall clock around each step).
roofline  the dominant kernel's algorithmic bytes per launch / its average
          CUDA-event duration in the timed region, against the measured HBM
          copy bandwidth.
cpu_baseline  the CPU oracle (the reference's algorithm restated in C, all
          host threads) on a bounded sample of the same workload.

The default run also measures the other configurations and adds them to
the headline line as sub-objects, each with its own value, e2e, roofline
and cpu_baseline: c1 (one 156-bead microtubule, 1e5 MD steps in one call,
CPU baseline over the whole run on all threads and on one), c2_batched_plain
(256 x 1520 beads), c3_ragged (the uneven 1024-trajectory batch) and
c4_tea_exact (16 x 3300 beads, exact TEA).  --no-suite skips them.

--impl reference times that CPU implementation alone: a port of the
reference's algorithm, not the reference program (its CUDA sources do not
travel to the GPU host, and its CPU-compilable kernel bodies cannot be built
there), labelled "kind": "port".

Multi-GPU (torchrun): each rank runs an independent copy of the workload
(trajectories are independent: replicas, no collective); value = all
ranks' monomer-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "monomer-steps/s on 1 GB300: exact TEA vs learned TEA at \u22641% mobility error"
UNIT = "monomer-steps/s"
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    # 256 trajectories of a 13 PF x 40 monomer lattice (520 beads) + 1000 free
    # tubulin monomers (500 dimers, GDP) in a 100 nm cube; Morse, 8 nm LJ list
    # rebuilt every 10 steps; no hydrodynamics.
    "batched_plain_256x1520": dict(kind="plain", ntraj=256, n_mon=40, n_free=1000, cube=100.0),
    # one straight 13 PF x 12 monomer lattice (156 beads, alternating alpha /
    # beta), no free tubulin, no hydrodynamics: 1e5 MD steps in one call,
    # pair lists rebuilt every 10 steps
    "single_156": dict(kind="long", ntraj=1, n_mon=12, n_free=0, cube=100.0, md_steps=100_000,
                       warm_md_steps=2_000),
    # small case for quick checks
    "plain_16x1520": dict(kind="plain", ntraj=16, n_mon=40, n_free=1000, cube=100.0),
    # uneven batch: 1024 trajectories, protofilament length U{8..120}, free
    # tubulin U{0..2000} in a 150 nm cube, 30% with a bent plus end
    # (0.1-0.3 rad per monomer); launch shapes from the autotuner
    "ragged_1024": dict(kind="plain", ragged=True, ntraj=1024, pf_range=(8, 120), free_range=(0, 2000), cube=150.0,
                        n_mon=64, n_free=1000),
    # exact TEA hydrodynamics: 16 trajectories of a 13 PF x 100 monomer lattice
    # (1300 beads) + 2000 free monomers; RPY radius 2 nm, epsilon/beta every
    # 10 steps (FP64 reduction on the device)
    "tea_exact_16x3300": dict(kind="tea", ntraj=16, n_mon=100, n_free=2000, cube=100.0),
    # exact TEA at the size of the learned-TEA comparison: 64 x (13 PF x 200 + 3000)
    "tea_exact_64x5600": dict(kind="tea", ntraj=64, n_mon=200, n_free=3000, cube=150.0),
    # learned vs exact TEA: the network is trained on 1e6 samples of the
    # 16 x 3300 exact-TEA system (Adam, batch 4096, 20 epochs), then both run
    # 64 x (13 PF x 200 + 3000) with an exact re-check every 100 steps
    "tea_learned_vs_exact_64x5600": dict(kind="tea_compare", ntraj=64, n_mon=200, n_free=3000, cube=150.0,
                                         train=dict(ntraj=16, n_mon=100, n_free=2000, cube=100.0),
                                         samples=1_000_000, epochs=20, batch=4096, lr=1e-3, recheck=100,
                                         max_err=0.01, theta=0.85, ff_refresh=1000),
    # stride-step work on the uneven batch: every 100 steps a DCD frame of
    # every trajectory, the energy totals, mt_length and hydrolysis; the
    # asynchronous pipeline and the device analytics against the reference's
    # synchronous download + host loops
    "stride_io_ragged_1024": dict(kind="stride", ragged=True, ntraj=1024, pf_range=(8, 120), free_range=(0, 2000),
                                  cube=150.0, n_mon=64, n_free=1000, stride=100),
}
DEFAULT_WORKLOAD = "tea_learned_vs_exact_64x5600"
# the other configurations, measured in the same default run and reported as
# sub-objects of the headline line
SUITE = (("c1", "single_156"), ("c2_batched_plain", "batched_plain_256x1520"), ("c3_ragged", "ragged_1024"),
         ("c4_tea_exact", "tea_exact_16x3300"))
SUB_KEYS = ("workload", "value", "unit", "ms_per_step", "steps", "warmup", "config", "roofline", "kernel_ms",
            "kernel_share", "dominant_kernel", "gpu_launches", "e2e", "clocks", "cpu_baseline")
PORT_NOTE = ("the oracle port: the reference's algorithm restated in C (oracle/), all host threads; the "
             "reference program itself is not timed (its CUDA sources do not travel to the GPU host and no "
             "aarch64 build of its CPU-compilable kernel bodies can be made here)")


# ---------------------------------------------------------------- helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Host-side barrier and max-reduction over ranks (gloo); no data-path collective."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the first sample before the timed region starts (nvidia-smi takes
            # a moment to come up), so that short regions are covered too
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.first = len(self.lines)
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        # one sample at or after the end of the timed region (200 ms period)
        n0, t0 = len(self.lines), time.time()
        while len(self.lines) == n0 and time.time() - t0 < 0.5 and self.proc.poll() is None:
            time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def workload_params(spec: dict, seed: int):
    from mt_gb300 import synth
    if spec["kind"] in ("tea", "tea_compare"):
        return synth.default_params(seed=seed, hdi_on=1, tea_a=2.0, tea_epsilon_freq=10)
    return synth.default_params(seed=seed)


def make_batch(spec: dict, seed: int, ntraj: int | None = None):
    from mt_gb300 import synth
    p = workload_params(spec, seed)
    if spec.get("ragged"):
        return synth.ragged_batch(p, ntraj or spec["ntraj"], seed=seed, pf_range=spec["pf_range"],
                                  free_range=spec["free_range"], cube=spec["cube"])
    return synth.uniform_batch(p, ntraj or spec["ntraj"], spec["n_mon"], spec["n_free"], seed=seed,
                               cube=spec["cube"])


TUNE_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "mt_gb300", "autotune.json")


def tune_key(b, workload: str) -> str:
    import torch
    return f"{torch.cuda.get_device_name()}|{workload}|nb={b.nbeads}|nt={b.ntraj}|tea={b.params.hdi_on}"


def tea_pairs(b) -> int:
    """Ordered non-extra pairs i != j per trajectory, summed: the TEA mobility product's units."""
    tot = 0
    for t in range(b.ntraj):
        n = int(np.count_nonzero(b.extra[b.offsets[t]:b.offsets[t + 1]] == 0))
        tot += n * (n - 1)
    return tot


def plain_step_time(kt_ms: dict, launches: dict, period: int):
    """(kernel, average device ms per MD step) of the plain path's step kernel:
    the per-step launch, or the persistent launch that covers a whole
    pair-list period of `period` steps."""
    if launches.get("step_period"):
        return "k_step_period", kt_ms["step_period"] / (launches["step_period"] * period)
    return "k_step_plain", kt_ms["step_plain"] / max(1, launches["step_plain"])


def ncu_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` recorded by an ncu capture summary under profiles/."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    d = json.load(open(path))
    return d.get(workload, {}).get(kernel)


# ------------------------------------------------------------ CPU baseline
def _omp_threads(n: int) -> bool:
    """Sets the OpenMP thread count of this process (the oracle's libgomp)."""
    import ctypes
    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(n))
        return True
    except (OSError, AttributeError):
        return False


def cpu_sample(spec: dict, seed: int, max_seconds: float = 20.0, single_core: bool = False):
    """Times the CPU oracle (all host threads) on a bounded sample: the first
    trajectories of the workload for one pair-list period (10 MD steps),
    doubling the sample until it takes a few seconds.  With single_core, one
    trajectory is also timed on one thread."""
    from mt_gb300 import synth
    from oracle import oracle
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
    o = oracle.Oracle("orc", "f32")

    def period_rate(ntr):
        b = make_batch(spec, seed, ntr)
        p = b.params
        seeds = o.generate_seeds(p.rseed, 2 * b.nbeads)
        period = int(p.ljpairsupdatefreq)
        t0 = time.perf_counter()
        o.run(b, b.coords, seeds, 0, period)
        dt = time.perf_counter() - t0
        return b.active_beads() * period / dt, dt, b.nbeads

    ntr = 1
    while True:
        rate, dt, nb = period_rate(ntr)
        if dt > 2.0 or ntr >= spec["ntraj"] or dt * 2 > max_seconds:
            break
        ntr *= 2
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    out = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{ntr} of {spec['ntraj']} trajectories ({nb} beads) x {10} MD steps (one list period), "
                     f"{dt:.2f} s", "note": PORT_NOTE}
    if single_core and _omp_threads(1):
        try:
            r1, dt1, nb1 = period_rate(1)
        finally:
            _omp_threads(cores)
        out["single_core"] = {"value": r1, "cores": 1,
                              "sample": f"1 trajectory ({nb1} beads) x 10 MD steps, {dt1:.2f} s"}
    return out


def cpu_full_run(spec: dict, seed: int):
    """The oracle port over the whole run of the single-trajectory
    configuration (all md_steps), on all host threads and on one thread."""
    from oracle import oracle
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
    o = oracle.Oracle("orc", "f32")
    b = make_batch(spec, seed)
    n = int(spec["md_steps"])
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))

    def rate():
        seeds = o.generate_seeds(b.params.rseed, 2 * b.nbeads)
        t0 = time.perf_counter()
        o.run(b, b.coords, seeds, 0, n)
        dt = time.perf_counter() - t0
        return b.active_beads() * n / dt, dt

    r_all, dt_all = rate()
    out = {"value": r_all, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"the whole run: {b.nbeads} beads x {n} MD steps, {dt_all:.2f} s", "note": PORT_NOTE}
    if _omp_threads(1):
        try:
            r1, dt1 = rate()
        finally:
            _omp_threads(cores)
        out["single_core"] = {"value": r1, "cores": 1, "sample": f"the whole run on one thread, {dt1:.2f} s"}
    return out


def run_reference(args, spec, dist):
    if dist.rank != 0:
        return
    seed = 1
    from mt_gb300 import synth
    from oracle import oracle
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
    o = oracle.Oracle("orc", "f32")
    # bounded per-step sample: as many trajectories as take ~1 s per period
    probe = cpu_sample(spec, seed, max_seconds=4.0)
    ntr = int(probe["sample"].split(" ")[0])
    b = make_batch(spec, seed, ntr)
    p = b.params
    seeds = o.generate_seeds(p.rseed, 2 * b.nbeads)
    period = int(p.ljpairsupdatefreq)
    x = b.coords
    ci = beta = None
    for w in range(args.warmup):
        x, _, seeds, _, _, ci, beta = o.run(b, x, seeds, w * period, period, tea_ci=ci, tea_beta=beta)
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        x, _, seeds, _, _, ci, beta = o.run(b, x, seeds, (args.warmup + k) * period, period, tea_ci=ci,
                                            tea_beta=beta)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = b.active_beads() * period * args.steps / tot
    cores = os.cpu_count() or 1
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": args.workload, "sample_trajectories": ntr, "md_steps_per_bench_step": period},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": int(os.environ.get("OMP_NUM_THREADS", cores)),
                            "kind": "port", "note": PORT_NOTE,
                            "sample": f"{ntr} of {spec['ntraj']} trajectories x {period} MD steps per bench step"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ------------------------------------------------------------------ main
def kernel_time_pass(e, step: int, period: int, nsteps: int, flush):
    """Per-kernel CUDA-event times from a second pass of the same steps (the
    timed pass runs without the per-kernel events, which would add gaps)."""
    import torch
    e.set_kernel_timing(True)
    e.step(step, period)          # captures the instrumented graph
    step += period
    e.kernel_times(reset=True)
    for _ in range(nsteps):
        flush.zero_()
        torch.cuda.synchronize()
        e.step_timed(step, period)
        step += period
    torch.cuda.synchronize()
    kt = e.kernel_times(reset=True)
    e.set_kernel_timing(False)
    e.step(step, period)          # the uninstrumented graph again
    step += period
    return step, kt


def run_gpu(args, spec, dist, cpu_seconds: float = 20.0):
    import torch

    from mt_gb300 import build as mbuild
    from mt_gb300 import engine

    mbuild.build()
    torch.cuda.set_device(dist.local)
    seed = 1 + dist.rank
    b = make_batch(spec, seed)
    b.params.device = dist.local
    e = engine.Engine(b)
    e.upload_state(b.coords)
    period = int(b.params.ljpairsupdatefreq)
    active = b.active_beads()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dist.local}")
    tune = e.autotune(0, period, cache=TUNE_CACHE, key=tune_key(b, args.workload))

    step = 0
    for _ in range(args.warmup):
        e.step(step, period)
        step += period
    e.graph_kernel_launches(reset=True)

    clocks = ClockSampler(dist.local)
    clocks.start()
    dist.barrier()
    ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ms.append(e.step_timed(step, period))
        step += period
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    graph_kernels = e.graph_kernel_launches(reset=True)   # every timed step is a graph replay
    step, kt = kernel_time_pass(e, step, period, args.steps, flush)
    total_ms = sum(ms)
    t_max = dist.max(total_ms)
    total_units = dist.sum(active * period * args.steps)
    value = total_units / (t_max / 1e3)

    kt_ms = {k: v[0] for k, v in kt.items()}
    launches = {k: v[1] for k, v in kt.items()}
    dominant = max(kt_ms, key=lambda k: kt_ms[k])
    if spec["kind"] == "plain":
        # list statistics for the algorithmic bytes of the fused step
        L = e.lists()
        n_i = (L["lj"][0].astype(np.int64) + L["long"][0] + L["lat"][0] + b.harmonic_count).astype(np.int64)
        act = b.extra == 0
        work = float(np.sum((48 + 64 + 16 + 4 * n_i)[act]))
        kname, avg_ms = plain_step_time(kt_ms, launches, period)
        peak, peak_kind = measured_peaks()
        achieved = work / (avg_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak,
                "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                "traffic": ncu_traffic(kname, args.workload), "algorithmic_bytes_per_md_step": work,
                "avg_ms_per_md_step": avg_ms}
    else:
        import ctypes as C
        work = 45.0 * tea_pairs(b)
        avg_ms = kt_ms["tea_step"] / max(1, launches["tea_step"])
        tf = C.c_double()
        engine.check(engine.load().mtg_measure_fp32_tflops(dist.local, C.byref(tf)))
        achieved = work / (avg_ms / 1e3) / 1e12
        roof = {"bound": "fp32", "kernel": "k_tea_step", "achieved": achieved, "peak": tf.value,
                "peak_source": "measured FP32 FMA rate (mtg_measure_fp32_tflops)", "unit": "TFLOP/s",
                "frac": achieved / tf.value, "traffic": ncu_traffic("k_tea_step", args.workload),
                "algorithmic_flop_per_launch": work, "avg_launch_ms": avg_ms}

    # end to end through the C ABI with pinned host buffers
    pin = engine.PinnedArray((e.nb, 7), np.float32)
    pin.array[:] = e.download_state()
    lib = engine.load()
    import ctypes as C
    fptr = pin.array.ctypes.data_as(C.POINTER(C.c_float))
    e2e_t = []
    for _ in range(max(3, args.steps)):
        t0 = time.perf_counter()
        engine.check(lib.mtg_upload_state(e.h, fptr))
        engine.check(lib.mtg_step(e.h, C.c_longlong(step), C.c_int(period)))
        engine.check(lib.mtg_download_state(e.h, fptr, C.cast(None, C.POINTER(C.c_float))))
        e2e_t.append(time.perf_counter() - t0)
        step += period
    e2e_max = dist.max(sum(e2e_t))
    e2e_value = dist.sum(active * period * len(e2e_t)) / e2e_max
    pin.free()

    out = None
    if dist.rank == 0:
        cpu = cpu_sample(spec, seed, max_seconds=cpu_seconds, single_core=True) \
            if dist.ws == 1 and not args.no_cpu_baseline else None
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "trajectories_per_gpu": b.ntraj, "beads_per_gpu": b.nbeads,
                       "active_beads_per_gpu": active, "md_steps_per_bench_step": period,
                       "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": f"replicas x{dist.ws} (independent trajectories)",
                       "tuning": tune},
            "roofline": roof,
            "kernel_ms": {k: (kt_ms[k] / launches[k] if launches[k] else None) for k in kt_ms},
            "kernel_share": {k: kt_ms[k] / max(1e-12, sum(kt_ms.values())) for k in kt_ms},
            "dominant_kernel": dominant,
            "gpu_launches": int(graph_kernels),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 28 * e.nb, "d2h_bytes_per_step": 28 * e.nb},
            "clocks": clk,
            "cpu_baseline": cpu,
        }
    e.close()
    return out


def run_long(args, spec, dist):
    """The single-microtubule configuration: one trajectory, all md_steps MD
    steps in one timed mtg_step call (graph replays of one pair-list period
    each), after warm_md_steps untimed steps; the per-kernel timing for the
    roofline comes from a separate 1000-step pass."""
    import torch

    from mt_gb300 import build as mbuild
    from mt_gb300 import engine

    mbuild.build()
    torch.cuda.set_device(dist.local)
    seed = 1 + dist.rank
    b = make_batch(spec, seed)
    b.params.device = dist.local
    e = engine.Engine(b)
    e.upload_state(b.coords)
    period = int(b.params.ljpairsupdatefreq)
    active = b.active_beads()
    n = int(spec["md_steps"])
    tune = e.autotune(0, period, cache=TUNE_CACHE, key=tune_key(b, args.workload))
    step = 0
    e.step(step, int(spec["warm_md_steps"]))
    step += int(spec["warm_md_steps"])
    e.set_kernel_timing(True)
    e.step(step, 1000)
    step += 1000
    e.kernel_times(reset=True)
    e.step(step, 1000)
    step += 1000
    kt = e.kernel_times(reset=True)
    e.set_kernel_timing(False)
    e.step(step, 1000)            # captures the untimed graphs again
    step += 1000
    e.graph_kernel_launches(reset=True)
    clocks = ClockSampler(dist.local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    ms = e.step_timed(step, n)
    step += n
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    launches_timed = e.graph_kernel_launches(reset=True)
    t_max = dist.max(ms)
    value = dist.sum(active * n) / (t_max / 1e3)
    kt_ms = {k: v[0] for k, v in kt.items()}
    nl = {k: v[1] for k, v in kt.items()}
    L = e.lists()
    n_i = (L["lj"][0].astype(np.int64) + L["long"][0] + L["lat"][0] + b.harmonic_count).astype(np.int64)
    work = float(np.sum((48 + 64 + 16 + 4 * n_i)[b.extra == 0]))
    kname, avg_ms = plain_step_time(kt_ms, nl, period)
    peak, peak_kind = measured_peaks()
    achieved = work / (avg_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "peak_source": peak_kind,
            "unit": "GB/s", "frac": achieved / peak, "traffic": None, "algorithmic_bytes_per_md_step": work,
            "avg_ms_per_md_step": avg_ms,
            "note": "156 beads: the working set (about 20 KB) stays on chip; each launch is bound by its "
                    "latency, not by HBM"}
    # end to end through the C ABI: upload from pinned memory, the whole run, download
    import ctypes as C
    pin = engine.PinnedArray((e.nb, 7), np.float32)
    pin.array[:] = e.download_state()
    lib = engine.load()
    fptr = pin.array.ctypes.data_as(C.POINTER(C.c_float))
    t0 = time.perf_counter()
    engine.check(lib.mtg_upload_state(e.h, fptr))
    engine.check(lib.mtg_step(e.h, C.c_longlong(step), C.c_int(n)))
    engine.check(lib.mtg_download_state(e.h, fptr, C.cast(None, C.POINTER(C.c_float))))
    e2e_s = dist.max(time.perf_counter() - t0)
    pin.free()
    out = None
    if dist.rank == 0:
        cpu = cpu_full_run(spec, seed) if dist.ws == 1 and not args.no_cpu_baseline else None
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws, "steps": 1, "warmup": 1,
               "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic",
               "config": {"workload": args.workload, "trajectories_per_gpu": b.ntraj, "beads_per_gpu": b.nbeads,
                          "active_beads_per_gpu": active, "md_steps_per_bench_step": n,
                          "warmup_md_steps": int(spec["warm_md_steps"]),
                          "l2": "not flushed: the 20 KB state is cache-resident by design",
                          "parallelism": f"replicas x{dist.ws} (independent trajectories)", "tuning": tune},
               "roofline": roof,
               "kernel_ms": {k: (kt_ms[k] / nl[k] if nl[k] else None) for k in kt_ms},
               "kernel_share": {k: kt_ms[k] / max(1e-12, sum(kt_ms.values())) for k in kt_ms},
               "dominant_kernel": max(kt_ms, key=lambda k: kt_ms[k]),
               "gpu_launches": int(launches_timed),
               "e2e": {"value": dist.sum(active * n) / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 28 * e.nb,
                       "d2h_bytes_per_step": 28 * e.nb},
               "clocks": clk, "cpu_baseline": cpu}
    e.close()
    return out


def run_suite_member(args, key: str, workload: str, dist):
    """One configuration of the default run's suite, as a sub-object."""
    import copy
    sub = copy.copy(args)
    sub.workload = workload
    spec = WORKLOADS[workload]
    if spec["kind"] == "long":
        r = run_long(sub, spec, dist)
    else:
        r = run_gpu(sub, spec, dist, cpu_seconds=6.0)
    if r is None:
        return None
    r = dict(r, workload=workload)
    return {k: r[k] for k in SUB_KEYS if k in r}


def tea_samples(tr: dict, device: int, seed: int, n: int, md_steps: int = 10_000):
    """(descriptor, C_i, beta) samples from an exact-TEA run of the system tr:
    snapshots spread evenly over md_steps MD steps (the 1e4 steps of the
    exact-TEA configuration) until n samples are collected."""
    from mt_gb300 import engine
    b = make_batch(tr, seed)
    b.params.device = device
    e = engine.Engine(b)
    e.upload_state(b.coords)
    snaps = -(-n // b.nbeads)
    every = max(10, md_steps // snaps // 10 * 10)
    Xs, Ts, step, k = [], [], 0, 0
    while k < n:
        e.step(step, every)
        step += every
        X, T = e.tea_training_data()
        Xs.append(X)
        Ts.append(T)
        k += len(X)
    e.close()
    return np.concatenate(Xs)[:n], np.concatenate(Ts)[:n], step


def train_surrogate(spec: dict, device: int, seed: int):
    """Exact-TEA runs of the training system -> (descriptor, C_i, beta) samples
    -> network; its error on held-out trajectories (another seed of the same
    system) against the mean predictor."""
    from mt_gb300 import engine
    tr = dict(spec["train"], kind="tea")
    t0 = time.perf_counter()
    X, T, steps = tea_samples(tr, device, seed + 1000, spec["samples"])
    t_data = time.perf_counter() - t0
    Xv, Tv, _ = tea_samples(tr, device, seed + 2000, 100_000, md_steps=2_000)
    s = engine.Surrogate(device=device, seed=seed)
    t0 = time.perf_counter()
    losses = s.train(X, T, epochs=spec["epochs"], batch=spec["batch"], lr=spec["lr"], seed=seed)
    t_train = time.perf_counter() - t0
    pred = s.predict(Xv)
    rms_net = np.sqrt(((pred - Tv) ** 2).mean(0)).tolist()
    rms_mean = np.sqrt(((T.mean(0) - Tv) ** 2).mean(0)).tolist()
    info = {"samples": int(len(X)), "md_steps_of_exact_tea": steps, "data_s": t_data, "train_s": t_train,
            "loss_first_epoch": float(losses[0]), "loss_last_epoch": float(losses[-1]),
            "held_out": f"{len(Xv)} samples of other trajectories of the training system",
            "rms_err_net_(Cx,Cy,Cz,beta)": rms_net, "rms_err_mean_predictor": rms_mean}
    return s, info


def tea_effective_error(e, recompute_exact: bool, farfield: bool):
    """RMS over active beads of |f - f_ref| / RMS |f_ref| for the effective TEA
    forces of the current state under one draw of F and R (the noise streams
    are restored, so both evaluations see the same R): f with the engine's
    current C_i and beta (and the far-field product when farfield), f_ref
    with freshly computed exact C_i and beta and the all-pairs product.
    Leaves the exact C_i and beta in the engine when recompute_exact."""
    seeds = e.download_rng()
    if farfield:
        _, f, _ = e.tea_effective_forces(exact=False, farfield=True)
    else:
        f, _, _ = e.tea_effective_forces(exact=True, farfield=False)
    e.upload_rng(seeds)
    if recompute_exact:
        e.tea_update()
    fr, _, _ = e.tea_effective_forces(exact=True, farfield=False)
    act = e.batch.extra == 0
    d = f[act, :3].astype(np.float64) - fr[act, :3]
    return float(np.sqrt((d ** 2).sum(1).mean() / (fr[act, :3].astype(np.float64) ** 2).sum(1).mean()))


def run_tea_compare(args, spec, dist):
    """Exact TEA, exact TEA with stale epsilon (recomputed once per re-check
    period, the zero-cost alternative to the network), and learned TEA (the
    network's C_i and beta, the far-field mobility product, the exact re-check
    every period) on the same batch, timed back to back."""
    import torch

    from mt_gb300 import build as mbuild
    from mt_gb300 import engine

    mbuild.build()
    torch.cuda.set_device(dist.local)
    seed = 1 + dist.rank
    surr, train_info = train_surrogate(spec, dist.local, seed)
    b = make_batch(spec, seed)
    b.params.device = dist.local
    period = int(spec["recheck"])
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dist.local}")
    active = b.active_beads()
    results = {}
    tune = None
    eps_freq = int(b.params.tea_epsilon_freq)
    for mode in ("exact", "exact_stale_eps", "learned"):
        b.params.tea_epsilon_freq = period if mode == "exact_stale_eps" else eps_freq
        e = engine.Engine(b)
        e.upload_state(b.coords)
        if mode == "exact":   # launch shapes from the autotuner (exact TEA), used by every path
            tune = e.autotune(0, 10, cache=TUNE_CACHE, key=tune_key(b, args.workload))
        else:
            e.set_tuning(**tune["tuning"])
        if mode == "learned":
            e.set_surrogate(surr, recheck_every=period, max_err=spec["max_err"])
            e.set_tea_farfield(True, spec["theta"], refresh_every=spec["ff_refresh"])
        step = 0
        for _ in range(args.warmup):
            e.step(step, period)
            step += period
        e.graph_kernel_launches(reset=True)
        clocks = ClockSampler(dist.local)
        clocks.start()
        dist.barrier()
        ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ms.append(e.step_timed(step, period))
            step += period
        dist.barrier()
        clk = clocks.stop()
        graph_kernels = e.graph_kernel_launches(reset=True)   # every timed step is a graph replay
        step, kt = kernel_time_pass(e, step, period, args.steps, flush)
        t_max = dist.max(sum(ms))
        value = dist.sum(active * period * args.steps) / (t_max / 1e3)
        res = {"value": value, "ms_per_step": t_max / args.steps, "clocks": clk,
               "kernel_ms": {k: (v[0] / v[1] if v[1] else None) for k, v in kt.items()},
               "kernel_share": {k: v[0] / max(1e-12, sum(x[0] for x in kt.values())) for k, v in kt.items()},
               "gpu_launches": int(graph_kernels), "kt": kt}
        if mode == "learned":
            res["status"] = e.surrogate_status()
            res["farfield"] = e.tea_farfield_stats()
        # e2e through the C ABI with pinned host buffers (one re-check period per step)
        import ctypes as C
        pin = engine.PinnedArray((e.nb, 7), np.float32)
        pin.array[:] = e.download_state()
        lib = engine.load()
        fptr = pin.array.ctypes.data_as(C.POINTER(C.c_float))
        tt = []
        for _ in range(max(2, args.steps)):
            t0 = time.perf_counter()
            engine.check(lib.mtg_upload_state(e.h, fptr))
            engine.check(lib.mtg_step(e.h, C.c_longlong(step), C.c_int(period)))
            engine.check(lib.mtg_download_state(e.h, fptr, C.cast(None, C.POINTER(C.c_float))))
            tt.append(time.perf_counter() - t0)
            step += period
        res["e2e"] = {"value": dist.sum(active * period * len(tt)) / dist.max(sum(tt)), "unit": UNIT,
                      "h2d_bytes_per_step": 28 * e.nb, "d2h_bytes_per_step": 28 * e.nb}
        pin.free()
        # errors of the effective TEA forces against fresh exact TEA, on these
        # (held-out) trajectories, at the end of a re-check period
        e.step(step, period - 1)
        step += period - 1
        if mode == "exact_stale_eps":     # C_i, beta from period - 1 steps ago
            res["mobility_error_vs_fresh_exact"] = tea_effective_error(e, True, False)
        if mode == "learned":             # the network's C_i, beta (all-pairs), then the far field alone
            res["mobility_error_network_only"] = tea_effective_error(e, True, False)
            res["mobility_error_farfield_only"] = tea_effective_error(e, False, True)
        e.close()
        results[mode] = res
    b.params.tea_epsilon_freq = eps_freq
    import ctypes as C
    tf = C.c_double()
    engine.check(engine.load().mtg_measure_fp32_tflops(dist.local, C.byref(tf)))

    def fp32_roof(kt, kind, kernel, work, note):
        avg = kt[kind][0] / max(1, kt[kind][1])
        ach = work / (avg / 1e3) / 1e12
        return {"bound": "fp32", "kernel": kernel, "achieved": ach, "peak": tf.value,
                "peak_source": "measured FP32 FMA rate (mtg_measure_fp32_tflops)", "unit": "TFLOP/s",
                "frac": ach / tf.value, "traffic": ncu_traffic(kernel, args.workload),
                "algorithmic_flop_per_launch": work, "avg_launch_ms": avg, "work": note}

    L, X, S = results["learned"], results["exact"], results["exact_stale_eps"]
    learned_ok = not L["status"]["fell_back"]
    ffs = L["farfield"]
    roof_exact = fp32_roof(X["kt"], "tea_step", "k_tea_step", 45.0 * tea_pairs(b), "45 FLOP per ordered pair")
    roof_ff = fp32_roof(L["kt"], "ff_near", "k_ff_near", 45.0 * ffs["near_pairs"],
                        "45 FLOP per ordered near pair (the pair loop of k_ff_near; its list walk not counted)")
    out = None
    if dist.rank == 0:
        cpu = cpu_sample(dict(spec, kind="tea"), seed, single_core=True) if dist.ws == 1 and not args.no_cpu_baseline else None
        out = {
            "metric": METRIC, "value": L["value"] if learned_ok else X["value"], "unit": UNIT, "n_gpus": dist.ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": L["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (network: bf16/f32)",
            "data": "synthetic",
            "config": {"workload": args.workload, "trajectories_per_gpu": b.ntraj, "beads_per_gpu": b.nbeads,
                       "md_steps_per_bench_step": period, "recheck_every": period, "max_mobility_error": spec["max_err"],
                       "farfield_theta": spec["theta"], "farfield_refresh_every": spec["ff_refresh"],
                       "tuning": tune,
                       "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": f"replicas x{dist.ws} (independent trajectories)"},
            "learned_tea": {"value": L["value"], "fell_back": not learned_ok,
                            "mobility_error_last_recheck": L["status"]["last_error"],
                            "mobility_error_network_only": L["mobility_error_network_only"],
                            "mobility_error_farfield_only": L["mobility_error_farfield_only"],
                            "rechecks": L["status"]["rechecks"], "farfield": ffs,
                            "ordered_pairs_all": tea_pairs(b), "kernel_ms": L["kernel_ms"],
                            "kernel_share": L["kernel_share"]},
            "exact_tea": {"value": X["value"], "ms_per_step": X["ms_per_step"], "kernel_ms": X["kernel_ms"],
                          "kernel_share": X["kernel_share"], "e2e": X["e2e"], "roofline": roof_exact},
            "exact_tea_stale_epsilon": {"value": S["value"], "ms_per_step": S["ms_per_step"],
                                        "epsilon_every": period,
                                        "mobility_error_vs_fresh_exact": S["mobility_error_vs_fresh_exact"],
                                        "kernel_ms": S["kernel_ms"]},
            "learned_over_exact": L["value"] / X["value"],
            "learned_over_exact_stale_epsilon": L["value"] / S["value"],
            "surrogate_training": train_info,
            "roofline": roof_ff,
            "gpu_launches": L["gpu_launches"],
            "e2e": L["e2e"] if learned_ok else X["e2e"],
            "clocks": L["clocks"],
            "cpu_baseline": cpu,
        }
    surr.close()
    return out


def run_stride(args, spec, dist):
    """Throughput with stride-step outputs: (a) mtg_output_frame (pinned
    double buffers + writer thread) and the device analytics (mt_length,
    hydrolysis) vs (b) the reference's order: synchronous download of the
    state and energies, host DCD writes, host mt_length / hydrolyse loops."""
    import tempfile

    import torch

    from mt_gb300 import build as mbuild
    from mt_gb300 import engine
    from oracle import dcd_oracle as D
    from oracle import updater_oracle as U

    mbuild.build()
    torch.cuda.set_device(dist.local)
    seed = 1 + dist.rank
    b = make_batch(spec, seed)
    b.params.device = dist.local
    stride = spec["stride"]
    active = b.active_beads()
    tmp = tempfile.mkdtemp(prefix="mtg_stride_")
    rng = np.random.default_rng(seed)
    res = {}
    for mode in ("async", "sync"):
        e = engine.Engine(b)
        e.upload_state(b.coords)
        e.autotune(0, 10, cache=TUNE_CACHE, key=tune_key(b, "ragged_1024"))
        xyz = [os.path.join(tmp, f"{mode}_xyz{t}.dcd") for t in range(b.ntraj)]
        ang = [os.path.join(tmp, f"{mode}_ang{t}.dcd") for t in range(b.ntraj)]
        nfile = args.warmup + args.steps
        if mode == "async":
            e.output_open(xyz, ang, nfile, 1, stride, float(b.params.dt), "REMARKS BENCH",
                          energy_path=os.path.join(tmp, "energies.txt"))
        else:
            for t in range(b.ntraj):
                n = int(b.offsets[t + 1] - b.offsets[t])
                for path in (xyz[t], ang[t]):
                    open(path, "wb").write(D.header(n, nfile, 1, stride, float(b.params.dt), "REMARKS BENCH"))
        on_cur = b.on_tubule.copy()
        gtp = b.gtp.copy()
        hook_s = []
        t0 = None
        for k in range(args.warmup + args.steps):
            if k == args.warmup:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
            e.step(k * stride, stride)
            h0 = time.perf_counter()
            if mode == "async":
                e.output_frame((k + 1) * stride, frame=True, energies=True)
                e.mt_length(save_prev=k > 0)
                n = e.hydrolysis_candidates()
                e.hydrolyse(rng.uniform(size=n))
            else:
                st = e.download_state()
                en = e.energies()
                for t in range(b.ntraj):
                    a, z = b.offsets[t], b.offsets[t + 1]
                    with open(xyz[t], "ab") as f:
                        f.write(D.frame(st[a:z, 0], st[a:z, 1], st[a:z, 2]))
                    with open(ang[t], "ab") as f:
                        f.write(D.frame(st[a:z, 3], st[a:z, 5], st[a:z, 4]))
                lines = "".join(f"Energies[{t}]:\t" + "\t".join(f"{v:f}" for v in u) + "\n" for t, u in enumerate(en))
                with open(os.path.join(tmp, "energies_sync.txt"), "a") as f:
                    f.write(lines)
                mt_len, on_new, on_prev = U.mt_length(st, b.offsets, on_cur, k > 0, on_cur)
                on_cur = on_new
                gtp, _ = U.hydrolyse_vec(b.offsets, gtp, b.extra, on_cur, on_prev, lambda m: rng.uniform(size=m))
                e.set_gtp(gtp)
                del lines, mt_len
            if k >= args.warmup:
                hook_s.append(time.perf_counter() - h0)
        if mode == "async":
            e.output_close()
        torch.cuda.synchronize()
        total = time.perf_counter() - t0
        res[mode] = {"value": active * stride * args.steps / total, "s_per_stride": total / args.steps,
                     "hook_ms_per_stride": 1e3 * float(np.mean(hook_s))}
        e.close()
    import shutil
    shutil.rmtree(tmp, ignore_errors=True)
    if dist.rank != 0:
        return None
    return {"metric": METRIC, "value": res["async"]["value"], "unit": UNIT, "n_gpus": dist.ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * res["async"]["s_per_stride"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "trajectories_per_gpu": b.ntraj, "beads_per_gpu": b.nbeads,
                       "md_steps_per_bench_step": stride,
                       "per_stride": "DCD frame of every trajectory (xyz + angles), energy totals, mt_length, "
                                     "hydrolysis"},
            "async_device_hooks": res["async"], "sync_host_hooks": res["sync"],
            "async_over_sync": res["async"]["value"] / res["sync"]["value"]}


# Small cases of the hot kernels for one-kernel ncu captures (`--profile-case`):
# each builds its system, runs a few warm-up launches and then `launches`
# launches of the kernel named, and prints one JSON line.  The command that
# captures one launch of, e.g., k_ff_near:
#   ncu --set full --clock-control none -k regex:k_ff_near -s 4 -c 1 -o prof \
#       python bench.py --profile-case ff_near
# Sizes are those of the workloads (one list period of steps, trajectories
# cut to keep a case at a few hundred MB on the device).
PROFILE_CASES = {
    # 16 of the 64 x 5600 learned-workload trajectories; untrained network
    # (the kernels' work does not depend on the weights), far field at the
    # workload's theta, no re-check
    "ff_near": dict(workload="tea_learned_vs_exact_64x5600", ntraj=16, steps=10),
    "tea_step": dict(workload="tea_exact_64x5600", ntraj=16, steps=10),
    "step_plain": dict(workload="ragged_1024", ntraj=None, steps=10),
    "step_period": dict(workload="single_156", ntraj=None, steps=100),
    # inference over the 16 x 5600 learned-workload beads, and one training
    # epoch (backward kernel) on their samples
    "mlp_infer": dict(workload="tea_learned_vs_exact_64x5600", ntraj=16, steps=6),
    "mlp_backward": dict(workload="tea_learned_vs_exact_64x5600", ntraj=16, steps=1),
}


def run_profile_case(name: str):
    c = PROFILE_CASES[name]
    spec = dict(WORKLOADS[c["workload"]])
    from mt_gb300 import build as mbuild
    from mt_gb300 import engine as eng

    mbuild.build()
    b = make_batch(spec, 1, c["ntraj"])
    out = {"profile_case": name, "workload": c["workload"], "trajectories": b.ntraj, "beads": b.nbeads}
    with eng.Engine(b) as e:
        e.upload_state(b.coords)
        if name in ("ff_near", "mlp_infer", "mlp_backward"):
            X, T = e.tea_training_data()
            s = eng.Surrogate(seed=1)
            if name == "mlp_backward":
                s.train(X, T, epochs=c["steps"], batch=spec["batch"], lr=spec["lr"], seed=1)
            elif name == "mlp_infer":
                for _ in range(c["steps"]):
                    s.predict(X)
            else:
                e.set_tuning(2, 128, 4, 1, plain_persistent=0)
                e.set_surrogate(s, recheck_every=0, max_err=1e9)
                e.set_tea_farfield(True, spec["theta"], refresh_every=spec["ff_refresh"])
                e.step(0, c["steps"])
                out["farfield"] = e.tea_farfield_stats()
            s.close()
        elif name == "step_period":
            e.set_tuning(2, 128, 8, 1, plain_persistent=1)
            e.step(0, c["steps"])
        else:
            if name == "step_plain":
                e.set_tuning(2, 256, 1, 1, plain_persistent=0)
            else:   # whole j ranges: k_tea_step alone, no split tail
                e.set_tuning(2, 128, 4, 1, plain_persistent=0)
            e.step(0, c["steps"])
        out["status"] = "ok"
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="mtg", choices=["mtg", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU-oracle sample (profiling runs)")
    ap.add_argument("--ff-theta", type=float, default=None,
                    help="admissibility of the learned mode's far field (default: the workload's)")
    ap.add_argument("--no-suite", action="store_true",
                    help="default workload only, without the other configurations' sub-objects")
    ap.add_argument("--profile-case", choices=sorted(PROFILE_CASES), default=None,
                    help="run one small case of a hot kernel for an ncu capture and exit")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args.profile_case)
        return
    spec = WORKLOADS[args.workload]
    if args.ff_theta is not None:
        spec = dict(spec, theta=args.ff_theta)
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dict(spec, kind="tea") if spec["kind"] == "tea_compare" else
                          dict(spec, kind="plain") if spec["kind"] in ("stride", "long") else spec, dist)
        elif spec["kind"] == "tea_compare":
            out = run_tea_compare(args, spec, dist)
            if args.workload == DEFAULT_WORKLOAD and not args.no_suite:
                for key, wl in SUITE:
                    r = run_suite_member(args, key, wl, dist)
                    if out is not None:
                        out[key] = r
            if out is not None:
                print(json.dumps(out))
        elif spec["kind"] == "long":
            out = run_long(args, spec, dist)
            if out is not None:
                print(json.dumps(out))
        elif spec["kind"] == "stride":
            out = run_stride(args, spec, dist)
            if out is not None:
                print(json.dumps(out))
        else:
            out = run_gpu(args, spec, dist)
            if out is not None:
                print(json.dumps(out))
    finally:
        dist.close()


if __name__ == "__main__":
    main()
