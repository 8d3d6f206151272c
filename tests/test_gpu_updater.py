"""Stride-step analytics on the device (mt_length, hydrolyse, change_conc's
counts and placements) against the CPU restatement of the reference's
updater (oracle/updater_oracle.py), through the C ABI."""
import numpy as np
import pytest

from helpers import small_system
from mt_gb300 import synth
from oracle import updater_oracle as U

pytestmark = pytest.mark.gpu


def batch_on_and_off_tubule(seed):
    """Lattice of radius 8.12 nm (on the tubule) plus free dimers, some of
    them placed inside the mt_length radius with tilted orientations."""
    b = small_system(seed=seed, ntr=3, n_mon=16, n_free=120, extra=2)
    rng = np.random.default_rng(seed)
    c = b.coords.copy()
    free = np.nonzero(b.fixed == 0)[0]
    pick = rng.choice(free, size=len(free) // 3, replace=False)
    c[pick, 0:2] = rng.uniform(-20, 20, size=(len(pick), 2))
    c[pick, 4] = rng.uniform(-2.0, 2.0, size=len(pick))   # theta
    return b, c


def margin_ok(c):
    return U.decision_margin(c).min() > 1e-4


def test_mt_length_matches_oracle(engine_mod):
    for seed in range(60, 80):
        b, c = batch_on_and_off_tubule(seed)
        if margin_ok(c):
            break
    e = engine_mod.Engine(b)
    e.upload_state(c)
    _, _, cur0, _ = e.download_flags()
    n0 = e.mt_length(save_prev=False)
    ref0, cur_ref, prev_ref = U.mt_length(c, b.offsets, cur0, False, np.zeros(b.nbeads, np.int32))
    assert np.array_equal(n0, ref0)
    _, _, cur, prev = e.download_flags()
    assert np.array_equal(cur, cur_ref)
    # second stride: prev takes the first result
    n1 = e.mt_length(save_prev=True)
    _, _, cur1, prev1 = e.download_flags()
    assert np.array_equal(prev1, cur_ref) and np.array_equal(cur1, cur_ref) and np.array_equal(n1, ref0)
    assert n0.sum() > 0 and n0.sum() < b.nbeads
    e.close()


def run_hydrolysis(engine_mod, b, c, gtp0, seed):
    e = engine_mod.Engine(b)
    e.upload_state(c)
    e.set_gtp(gtp0)
    e.mt_length(save_prev=False)
    e.mt_length(save_prev=True)            # on_cur = on_prev = the current test
    gtp_d, extra_d, cur, prev = e.download_flags()
    n = e.hydrolysis_candidates()
    rng = np.random.default_rng(seed)
    prob = rng.uniform(0.0, 0.05, size=n)  # many below 0.02
    nh, nr, ev = e.hydrolyse(prob, events=True)
    gtp_after, _, _, _ = e.download_flags()
    e.close()
    it = iter(prob)
    ref_gtp, draws, ref_ev = U.hydrolyse(b.offsets, gtp_d, extra_d, cur, prev, lambda: next(it))
    return n, draws, gtp_after, ref_gtp, nh, nr, ev, ref_ev


def test_hydrolyse_matches_oracle(engine_mod):
    b, c = batch_on_and_off_tubule(61)
    gtp0 = np.where(np.arange(b.nbeads) % 4 < 2, 1, 0).astype(np.int32)
    n, draws, got, ref, nh, nr, ev, ref_ev = run_hydrolysis(engine_mod, b, c, gtp0, 7)
    assert n == draws and n > 0
    assert np.array_equal(got, ref)
    assert nh == sum(1 for v in ref_ev.values() if v == 1) and nh > 0
    assert nr == sum(1 for v in ref_ev.values() if v == 2) and nr > 0
    for (k, t), v in ref_ev.items():
        assert ev[k, t] == v
    assert int(np.count_nonzero(ev)) == len(ref_ev)


def test_hydrolyse_ragged_matches_oracle(engine_mod):
    p = synth.default_params(seed=62)
    b = synth.ragged_batch(p, 6, seed=62, pf_range=(8, 20), free_range=(0, 200), cube=60.0, radius=8.12)
    c = b.coords.copy()
    gtp0 = np.ones(b.nbeads, np.int32)
    n, draws, got, ref, nh, nr, ev, ref_ev = run_hydrolysis(engine_mod, b, c, gtp0, 8)
    assert n == draws and np.array_equal(got, ref)


def test_count_extra_and_set_beads(engine_mod):
    b = small_system(seed=63, extra=3)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    assert np.array_equal(e.count_extra(), U.count_extra(b.offsets, b.extra))
    # change_conc re-inserts an extra dimer: two beads get new coordinates and extra = 0
    idx = np.nonzero(b.extra)[0][:2]
    new = b.coords[idx].copy()
    new[:, 0:3] = [[1.0, 2.0, 30.0], [1.0, 2.0, 34.0]]
    e.set_beads(idx, new, extra=np.zeros(2, np.uint8))
    st = e.download_state()
    assert np.array_equal(st[idx, :6], new[:, :6])
    ref_extra = b.extra.copy()
    ref_extra[idx] = 0
    assert np.array_equal(e.count_extra(), U.count_extra(b.offsets, ref_extra))
    _, x, _, _ = e.download_flags()
    assert np.array_equal(x, ref_extra)
    e.close()
