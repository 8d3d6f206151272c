"""GPU parity on the benchmarked workloads: trajectories generated exactly as
bench.py generates them (12 nm lattice with all angles 0, free dimers with
U[-pi, pi) angles in a 100 or 150 nm cube), at the trajectory sizes the bench
times: 1520 beads (batched plain), up to 3560 beads (uneven batch), 3300
beads (exact TEA) and 5600 beads (learned vs exact TEA).  The CUDA path
(through the C ABI) is compared with the FP32 oracle per bead, and both with
the FP64 oracle, on identical states and noise streams.

Bars, per bead (row norms of 3-vectors), each error taken relative to
max(|ref_i|, FLOOR x RMS over beads of |ref|) with FLOOR = 1: a max-norm at
the array's own scale, so that no bead can hide in an array norm, while
beads whose value nearly cancels (a bond at rest: the difference of two
coordinates near 100 nm, where one FP32 ulp is 8e-6 nm) are held to the
array's scale rather than to their own rounding noise.  The FP32 oracle
itself differs from the FP64 one by up to 1e-2 of |f_i| on such beads; the
errors at a floor of 1e-3 x RMS are recorded beside the bar for that reason:
* LJ lists bit-exact (centre distances are correctly rounded on both sides);
  longitudinal/lateral lists bit-exact except where the FP64 site distance of
  a pair lies within TIE nm of the 2.5 nm cutoff (sin/cos differ by an ulp);
* forces, per-bead energies, TEA C_i: <= RTOL relative to the FP32 oracle,
  plus the FP32 rounding envelope 2 E32, E32 = the FP32 oracle's own largest
  absolute error against the FP64 oracle over the array.  The envelope only
  matters where a value is rounding noise: the translational force of a
  bead of a straight lattice at rest, or of a free dimer whose bond sits at
  its rest length (the sine and cosine of its random angles round by an ulp
  differently in CUDA and in libm, and C = 300 kcal/mol/nm^2 turns that into
  about 1e-4 of force), and the lateral Morse energy per bead (one ulp of D).
  Everywhere else RTOL alone decides (the recorded gpu_vs_fp32_oracle);
* per-trajectory energy totals, epsilon and beta: <= RTOL relative;
* one step (plain or TEA) from identical state and seeds: noise streams
  bit-exact, every coordinate within 2 FP32 ulps of its value + RTOL x the
  RMS displacement of the step, against the FP32 oracle (the Gaussian
  deviates use the hardware sine, cosine and logarithm as the reference's
  GPU build does, the oracle uses libm as the reference's CPU build of the
  same kernels does: about 1e-6 apart per deviate);
* the GPU's largest error against the FP64 oracle stays within twice the
  FP32 oracle's own largest error against it (plus RTOL x RMS).
The errors against both oracles are recorded per quantity; with
MTG_PARITY_REPORT=<path> they are written there as JSON.
"""
import json
import os
import sys

import numpy as np
import pytest

from helpers import per_bead_rel, site_tie_distance, ulp32

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

RTOL = 1e-5
FLOOR = 1.0
FLOOR_INFO = 1e-3
TIE = 1e-4
REPORT = {}


@pytest.fixture(scope="module", autouse=True)
def _write_report():
    yield
    path = os.environ.get("MTG_PARITY_REPORT")
    if path and REPORT:
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "w") as f:
            json.dump({"rtol": RTOL, "floor_of_rms": FLOOR, "tie_nm": TIE, "cases": REPORT}, f, indent=1,
                      sort_keys=True)


def envelope_check(got, o32, o64, act):
    """Largest per-bead |got - o32| in units of RTOL max(|o32_i|, RMS) + 2 E32
    (<= 1 passes), and E32 relative to the RMS."""
    got, o32, o64 = (np.asarray(a, np.float64)[act] for a in (got, o32, o64))
    if got.ndim == 1:
        got, o32, o64 = got[:, None], o32[:, None], o64[:, None]
    mag = np.linalg.norm(o32, axis=1)
    rms = float(np.sqrt(np.mean(mag ** 2))) if len(mag) else 0.0
    e32 = float(np.max(np.linalg.norm(o32 - o64, axis=1), initial=0.0))
    tol = RTOL * np.maximum(mag, FLOOR * rms) + 2 * e32
    d = np.linalg.norm(got - o32, axis=1)
    return float(np.max(d / np.maximum(tol, 1e-300), initial=0.0)), e32 / max(rms, 1e-300)


def record(case, quantity, **vals):
    REPORT.setdefault(case, {})[quantity] = {k: (float(v) if isinstance(v, (float, np.floating)) else v)
                                            for k, v in vals.items()}


def bench_batch(workload, ntraj, seed=1, tea=None):
    import bench
    spec = dict(bench.WORKLOADS[workload])
    if tea is not None:
        spec["kind"] = "tea" if tea else "plain"
    return bench.make_batch(spec, seed, ntraj)


def uneven_batch(seed=3):
    """Three trajectories of the uneven workload's generator: the largest
    lattice (13 x 120) with the most free tubulin (2000) and a bent plus end,
    the smallest lattice (13 x 8) without free tubulin, and one between."""
    from mt_gb300 import synth
    p = synth.default_params(seed=seed)
    trajs = [synth.make_trajectory(120, 2000, seed=seed, cube=150.0, tail=6, bend=0.25),
             synth.make_trajectory(8, 0, seed=seed + 1, cube=150.0),
             synth.make_trajectory(64, 1000, seed=seed + 2, cube=150.0, tail=6, bend=0.1)]
    return synth.batch_from_trajectories(p, trajs)


CASES = {
    "batched_plain_256x1520": lambda: bench_batch("batched_plain_256x1520", 2),
    "ragged_1024": uneven_batch,
    "tea_exact_16x3300": lambda: bench_batch("tea_exact_16x3300", 2, tea=False),
    "tea_learned_vs_exact_64x5600": lambda: bench_batch("tea_exact_64x5600", 2, tea=False),
}


def compare_lists(case, e, L, b):
    got = {k: e.list_of_lists(k) for k in ("lj", "long", "lat")}
    want = {k: L.as_lists(k) for k in ("lj", "long", "lat")}
    assert got["lj"] == want["lj"], "LJ lists differ"
    ties, bad = 0, []
    for k in ("long", "lat"):
        for g in range(b.nbeads):
            if got[k][g] != want[k][g]:
                if site_tie_distance(b, b.coords, g) < TIE:
                    ties += 1
                else:
                    bad.append((k, g, got[k][g], want[k][g]))
    record(case, "lists", lj_entries=int(sum(len(x) for x in want["lj"])),
           long_entries=int(sum(len(x) for x in want["long"])), lat_entries=int(sum(len(x) for x in want["lat"])),
           beads_differing_at_a_tie=ties)
    assert not bad, bad[:5]
    return ties


@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("case", list(CASES))
def test_lists_forces_energies_on_bench_workloads(engine_mod, oracle_lib, case, method):
    b = CASES[case]()
    o32, o64 = oracle_lib.Oracle("orc", "f32"), oracle_lib.Oracle("orc", "f64")
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.set_list_method(method)
    e.rebuild_pairs()
    L = o32.lists(b, b.coords)
    ties = compare_lists(f"{case}/list_method_{method}", e, L, b)
    f = e.compute_forces()
    fo, f64 = o32.forces(b, b.coords, L), o64.forces(b, b.coords, L)
    act = b.extra == 0
    if ties:   # beads whose lists differ at a tie have different forces by construction
        gl, gt, wl, wt = e.list_of_lists("long"), e.list_of_lists("lat"), L.as_lists("long"), L.as_lists("lat")
        same = np.array([gl[g] == wl[g] and gt[g] == wt[g] for g in range(b.nbeads)])
        act = act & same
    name = f"{case}/list_method_{method}"
    for q, cols in (("force_translational", slice(0, 3)), ("force_angular", slice(3, 6))):
        e32, rms = per_bead_rel(f[:, cols], fo[:, cols], act, FLOOR)
        e64, _ = per_bead_rel(f[:, cols], f64[:, cols], act, FLOOR)
        o_64, _ = per_bead_rel(fo[:, cols], f64[:, cols], act, FLOOR)
        i32, _ = per_bead_rel(f[:, cols], fo[:, cols], act, FLOOR_INFO)
        i64, _ = per_bead_rel(f[:, cols], f64[:, cols], act, FLOOR_INFO)
        io64, _ = per_bead_rel(fo[:, cols], f64[:, cols], act, FLOOR_INFO)
        env, e32_rel = envelope_check(f[:, cols], fo[:, cols], f64[:, cols], act)
        record(name, q, gpu_vs_fp32_oracle=e32, gpu_vs_fp64_oracle=e64, fp32_oracle_vs_fp64=o_64, rms=rms,
               beads=int(act.sum()), at_floor_1e3_gpu_vs_fp32=i32, at_floor_1e3_gpu_vs_fp64=i64,
               at_floor_1e3_fp32_vs_fp64=io64, fp32_envelope_of_rms=e32_rel, envelope_ratio=env)
        assert env <= 1.0, (q, e32, e64, o_64, env)
        assert e64 <= 2 * o_64 + RTOL, (q, e64, o_64)
    tot, per = e.energies(per_bead=True)
    eo, e64o = o32.energies(b, b.coords, L), o64.energies(b, b.coords, L)
    terms = ("U_harm", "U_long", "U_lat", "U_psi", "U_fi", "U_teta", "U_lj")
    for c, q in enumerate(terms):
        e32, rms = per_bead_rel(per[:, c], eo[:, c], act, FLOOR)
        e64, _ = per_bead_rel(per[:, c], e64o[:, c], act, FLOOR)
        i32, _ = per_bead_rel(per[:, c], eo[:, c], act, FLOOR_INFO)
        env, e32_rel = envelope_check(per[:, c], eo[:, c], e64o[:, c], act)
        record(name, f"energy_per_bead_{q}", gpu_vs_fp32_oracle=e32, gpu_vs_fp64_oracle=e64, rms=rms,
               at_floor_1e3_gpu_vs_fp32=i32, fp32_envelope_of_rms=e32_rel, envelope_ratio=env)
        assert env <= 1.0, (q, e32, env)
    # per-trajectory totals: the sum of the per-bead allowances above bounds them
    for t in range(b.ntraj):
        sl = slice(int(b.offsets[t]), int(b.offsets[t + 1]))
        ref32, ref64 = eo[sl].sum(0), e64o[sl].sum(0)
        scale = np.maximum(np.abs(ref32), FLOOR_INFO * np.abs(ref32).max())
        r32 = float(np.max(np.abs(tot[t] - ref32) / scale))
        r64 = float(np.max(np.abs(tot[t] - ref64) / scale))
        a = act[sl]
        v32, v64 = eo[sl][a], e64o[sl][a]
        rms = np.sqrt((v32 ** 2).mean(0))
        allow = (RTOL * np.maximum(np.abs(v32), FLOOR * rms)).sum(0) + 2 * np.abs(v32 - v64).max(0) * a.sum()
        ratio = float(np.max(np.abs(tot[t] - ref32) / np.maximum(allow, 1e-300)))
        record(name, f"energy_totals_traj{t}", gpu_vs_fp32_oracle=r32, gpu_vs_fp64_oracle=r64,
               allowance_ratio=ratio)
        if not ties:
            assert ratio <= 1.0, (t, r32, ratio)
    e.close()


def step_errors(x, xo, x0):
    """Largest excess of |x - xo| over 2 FP32 ulps of xo, relative to
    max(|xo - x0|, FLOOR x RMS displacement) (per coordinate, 6 DOF), and
    the largest |x - xo| in nm / rad."""
    x, xo, x0 = (np.asarray(a, np.float64)[:, :6] for a in (x, xo, x0))
    disp = np.abs(xo - x0)
    excess = np.maximum(np.abs(x - xo) - 2 * ulp32(xo), 0.0)
    return float(np.max(excess / np.maximum(disp, FLOOR * np.sqrt(np.mean(disp ** 2))))), \
        float(np.max(np.abs(x - xo)))


@pytest.mark.parametrize("case", ["batched_plain_256x1520", "ragged_1024"])
def test_one_plain_step_on_bench_workloads(engine_mod, oracle_lib, case):
    b = CASES[case]()
    o32, o64 = oracle_lib.Oracle("orc", "f32"), oracle_lib.Oracle("orc", "f64")
    seeds = o32.generate_seeds(b.params.rseed, 2 * b.nbeads)
    xo, _, so, Lo, st, _, _ = o32.run(b, b.coords, seeds, 0, 1)
    x64 = o64.run(b, b.coords, seeds, 0, 1)[0]
    assert st == 0
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.step(0, 1)
    x = e.download_state()
    assert np.array_equal(e.download_rng(), so)
    err32, abs32 = step_errors(x, xo, b.coords)
    err64, abs64 = step_errors(x, x64, b.coords)
    record(case, "one_step_state", gpu_vs_fp32_oracle=err32, gpu_vs_fp64_oracle=err64,
           max_abs_nm_vs_fp32=abs32, max_abs_nm_vs_fp64=abs64)
    assert err32 <= RTOL, (err32, abs32)
    e.close()


@pytest.mark.parametrize("case", ["tea_exact_16x3300", "tea_learned_vs_exact_64x5600"])
def test_tea_on_bench_workloads(engine_mod, oracle_lib, case):
    """epsilon, beta and C_i, then one TEA step with the whole j range per
    CTA and with split j ranges (the split tail and the near-field rescan of
    the all-pairs kernels), against the oracle at the bench's trajectory size."""
    b = CASES[case]()
    b.params.hdi_on = 1
    b.params.tea_a = 2.0
    b.params.tea_epsilon_freq = 10
    from mt_gb300 import synth
    synth.derive_params(b.params)
    o32, o64 = oracle_lib.Oracle("orc", "f32"), oracle_lib.Oracle("orc", "f64")
    act = b.extra == 0
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    eps, beta, ci, rc = e.tea_update()
    assert rc == 0
    ci_o, eps_o = o32.tea_epsilon(b, b.coords)
    eps_t, beta_o, st = o32.tea_beta(b, eps_o)
    ci_64, eps_64 = o64.tea_epsilon(b, b.coords)
    eps_t64, beta_64, _ = o64.tea_beta(b, eps_64)
    e32, rms = per_bead_rel(ci[:, :3], ci_o[:, :3], act, FLOOR)
    e64, _ = per_bead_rel(ci[:, :3], ci_64[:, :3], act, FLOOR)
    record(case, "tea_ci", gpu_vs_fp32_oracle=e32, gpu_vs_fp64_oracle=e64, rms=rms)
    assert e32 <= RTOL, e32
    r_eps = float(np.max(np.abs(eps - eps_t) / np.abs(eps_t)))
    r_beta = float(np.max(np.abs(beta - beta_o) / np.abs(beta_o)))
    record(case, "tea_epsilon", gpu_vs_fp32_oracle=r_eps,
           gpu_vs_fp64_oracle=float(np.max(np.abs(eps - eps_t64) / np.abs(eps_t64))))
    record(case, "tea_beta", gpu_vs_fp32_oracle=r_beta,
           gpu_vs_fp64_oracle=float(np.max(np.abs(beta - beta_64) / np.abs(beta_64))))
    assert r_eps <= RTOL and r_beta <= RTOL, (r_eps, r_beta)
    e.close()
    seeds = o32.generate_seeds(b.params.rseed, 2 * b.nbeads)
    xo, _, so, _, st, _, _ = o32.run(b, b.coords, seeds, 0, 1)
    x64 = o64.run(b, b.coords, seeds, 0, 1)[0]
    assert st == 0
    for slices, jp in ((1, 1), (4, 4)):
        e2 = engine_mod.Engine(b)
        e2.upload_state(b.coords)
        t = e2.tuning()
        e2.set_tuning(t["list_method"], t["step_block"], slices, jp)
        e2.step(0, 1)
        assert np.array_equal(e2.download_rng(), so)
        x = e2.download_state()
        err32, abs32 = step_errors(x, xo, b.coords)
        err64, abs64 = step_errors(x, x64, b.coords)
        record(case, f"tea_step_state_slices{slices}_jparts{jp}", gpu_vs_fp32_oracle=err32,
               gpu_vs_fp64_oracle=err64, max_abs_nm_vs_fp32=abs32, max_abs_nm_vs_fp64=abs64)
        assert err32 <= RTOL, (slices, jp, err32, abs32)
        e2.close()
