"""The far field of the learned TEA mobility product on the GPU
(mtg_set_tea_farfield): its kernels against the FP64 restatement
(oracle/tea_ff_oracle.py) on the engine's own tree, its approximation
error against the exact all-pairs product at the learned comparison's
trajectory size (5600 beads), and the learned mode running with it: re-checks
against exact TEA, the fall-back to the exact product bit for bit, and the
periodic rebuild of the grouping."""
import os
import sys

import numpy as np
import pytest

from helpers import per_bead_rel, small_system

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

RTOL = 1e-5
THETA = 0.85


def tea_batch(ntraj=2, seed=1):
    """Trajectories of the learned-vs-exact workload: 13 PF x 200 lattice +
    3000 free monomers in a 150 nm cube, TEA on (a = 2 nm, epsilon every 10)."""
    import bench
    return bench.make_batch(dict(bench.WORKLOADS["tea_exact_64x5600"]), seed, ntraj)


def bead_traj(b):
    return np.repeat(np.arange(b.ntraj), np.diff(b.offsets))


def test_farfield_kernels_match_fp64_restatement(engine_mod):
    from oracle import tea_ff_oracle as O
    b = tea_batch()
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    eps, beta, ci, rc = e.tea_update()
    assert rc == 0
    e.set_tea_farfield(True, THETA)
    st = e.tea_farfield_stats()
    layout = e.tea_farfield_layout()
    leaf_start, leaf_bead, _, _, node_range, node_parent, far_start, _ = layout
    nleaf = len(leaf_start) - 1
    assert np.all(np.diff(leaf_start) <= 32) and np.all(np.diff(leaf_start) > 0)
    act = b.extra == 0
    assert sorted(leaf_bead.tolist()) == np.nonzero(act)[0].tolist()   # every active bead in one leaf
    assert np.array_equal(node_range[0:2 * nleaf:2], leaf_start[:-1])
    assert np.all(node_parent[nleaf:] < np.arange(nleaf, len(node_parent)))   # larger nodes first
    assert (np.diff(far_start)[nleaf:] > 0).any()                      # internal nodes take part
    fe, ff, rf = e.tea_effective_forces()
    _, F = e.download_state(forces=True)
    betab = beta[bead_traj(b)]
    ref_ff = O.effective_forces(b.coords, F, rf, ci, betab, b.params.tea_a, layout)
    err_ff, rms = per_bead_rel(ff[:, :3], ref_ff, act, 1.0)
    assert err_ff <= RTOL, err_ff
    ref_ex = np.zeros_like(ref_ff)
    for t in range(b.ntraj):
        beads = np.arange(b.offsets[t], b.offsets[t + 1])
        beads = beads[act[beads]]
        ref_ex[beads] = O.exact_effective_forces(b.coords, F, rf, ci, betab, b.params.tea_a, beads)[beads]
    err_ex, _ = per_bead_rel(fe[:, :3], ref_ex, act, 1.0)
    assert err_ex <= RTOL, err_ex
    # the approximation itself: RMS difference relative to the exact effective forces
    d = ff[act, :3].astype(np.float64) - fe[act, :3]
    approx = float(np.sqrt((d ** 2).sum(1).mean() / (fe[act, :3].astype(np.float64) ** 2).sum(1).mean()))
    assert approx < 5e-3, approx
    # the work it saves: bead pairs summed exactly and proxy pairs against all ordered pairs
    n = np.diff(b.offsets)
    allpairs = int((n * (n - 1)).sum())
    assert st["near_pairs"] + 2 * st["proxy_pairs"] < 0.5 * allpairs, (st, allpairs)
    e.close()


def _trained_surrogate(engine_mod):
    from test_gpu_surrogate import tea_dataset
    X, T = tea_dataset(engine_mod, seed=51)
    s = engine_mod.Surrogate(seed=11)
    s.train(X, T, epochs=40, batch=512, lr=2e-3, seed=3)
    return s


def test_learned_mode_with_farfield_runs_and_rechecks(engine_mod):
    s = _trained_surrogate(engine_mod)
    from mt_gb300 import synth
    p = synth.default_params(seed=52, hdi_on=1, tea_epsilon_freq=5)
    b = synth.uniform_batch(p, 3, 60, 900, seed=52, cube=80.0, thermal=0.05, n_extra_dimers=2)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.set_surrogate(s, recheck_every=10, max_err=1.0)
    e.set_tea_farfield(True, THETA, refresh_every=15)
    e.set_kernel_timing(True)
    e.step(0, 30)                   # rebuilds the grouping after step 15
    kt = e.kernel_times()
    st = e.surrogate_status()
    assert not st["fell_back"] and st["rechecks"] == 3, st
    # a network trained on 20-monomer systems, run on 60-monomer ones: the
    # bench measures the accuracy of a network trained for its workload
    assert np.isfinite(st["last_error"]) and st["last_error"] < 0.1, st
    assert kt["ff_near"][1] >= 10 and kt["ff_far"][1] >= 10 and kt["ff_proxies"][1] >= 10
    assert kt["tea_step"][0] < kt["ff_near"][0]
    x = e.download_state()
    assert np.all(np.isfinite(x))
    extra = b.extra.astype(bool)
    assert np.array_equal(x[extra], b.coords[extra])     # extra beads stay where they are
    e.close()


def test_farfield_fallback_reproduces_exact_tea(engine_mod):
    """max_err = 0: the first re-check falls back, and from then on the gated
    exact product runs: the run equals the exact-TEA run bit for bit."""
    b = small_system(seed=53, ntr=2, n_mon=30, n_free=300, tea=True, tea_epsilon_freq=5)
    s = engine_mod.Surrogate(seed=12)
    e1 = engine_mod.Engine(b)
    e1.upload_state(b.coords)
    e1.set_surrogate(s, recheck_every=10, max_err=0.0)
    e1.set_tea_farfield(True, THETA)
    e1.step(0, 20)
    assert e1.surrogate_status()["fell_back"]
    e2 = engine_mod.Engine(b)
    e2.upload_state(b.coords)
    e2.step(0, 20)
    assert np.array_equal(e1.download_state(), e2.download_state())
    assert np.array_equal(e1.download_rng(), e2.download_rng())


def test_farfield_graph_replay_equals_single_steps(engine_mod):
    s = _trained_surrogate(engine_mod)
    b = small_system(seed=54, ntr=2, n_mon=30, n_free=300, tea=True, tea_epsilon_freq=5)
    runs = []
    for chunk in (20, 1):
        e = engine_mod.Engine(b)
        e.upload_state(b.coords)
        e.set_surrogate(s, recheck_every=10, max_err=1.0)
        e.set_tea_farfield(True, THETA)
        for k in range(0, 20, chunk):
            e.step(k, chunk)
        runs.append((e.download_state(), e.download_rng()))
        e.close()
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


def test_farfield_rejects_bad_arguments(engine_mod):
    b = small_system(seed=55)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    with pytest.raises(engine_mod.MtgError, match="hdi_on"):
        e.set_tea_farfield(True, THETA)
    e.close()
    bt = small_system(seed=55, tea=True)
    e = engine_mod.Engine(bt)
    e.upload_state(bt.coords)
    with pytest.raises(engine_mod.MtgError, match="theta"):
        e.set_tea_farfield(True, 1.5)
    e.close()
