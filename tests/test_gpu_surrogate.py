"""Learned TEA on the GPU: the hand-written BF16 tensor-core forward/backward
against the FP64 CPU oracle, training, the gain over the method without the
network, and the learned mode of the step loop with its exact re-check."""
import numpy as np
import pytest

from helpers import small_system
from mt_gb300 import synth
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def layer_slices():
    return {"w1": slice(M.OFF_W1, M.OFF_W2), "w2": slice(M.OFF_W2, M.OFF_W3), "w3": slice(M.OFF_W3, M.OFF_W4),
            "w4": slice(M.OFF_W4, M.OFF_B), "b": slice(M.OFF_B, M.NPARAMS)}


def test_gradients_match_cpu_oracle(engine_mod):
    rng = np.random.default_rng(3)
    s = engine_mod.Surrogate(seed=5)
    X = rng.normal(2.0, 1.5, size=(384, M.IN)).astype(np.float32)
    T = rng.normal(0.9, 0.05, size=(384, M.OUT)).astype(np.float32)
    norm = np.concatenate([X.mean(0), 1 / X.std(0), T.mean(0), T.std(0)]).astype(np.float32)
    s.set_params(norm=norm)
    p, nrm = s.params()
    loss, g = s.loss_grad(X, T)
    Xn, Tn = M.normalise(X, T, nrm)
    l_emul, g_emul = M.loss_grad(p, Xn, Tn, emulate_bf16=True)
    l_exact, g_exact = M.loss_grad(p, Xn, Tn, emulate_bf16=False)
    assert abs(loss - l_emul) / l_emul < 2e-3
    for name, sl in layer_slices().items():
        err = np.linalg.norm(g[sl] - g_emul[sl]) / np.linalg.norm(g_emul[sl])
        err64 = np.linalg.norm(g[sl] - g_exact[sl]) / np.linalg.norm(g_exact[sl])
        assert err < 2e-2, (name, err)       # against the BF16-emulating oracle
        assert err64 < 6e-2, (name, err64)   # against exact FP64 (BF16 rounding of the inputs)


def test_predict_matches_cpu_oracle(engine_mod):
    rng = np.random.default_rng(4)
    s = engine_mod.Surrogate(seed=6)
    X = rng.normal(size=(300, M.IN)).astype(np.float32)
    p, nrm = s.params()
    Xn, _ = M.normalise(X, np.zeros((300, M.OUT)), nrm)
    y_ref, _ = M.forward(p, Xn, emulate_bf16=True)
    y = s.predict(X)
    y_ref = y_ref * nrm[2 * M.IN + M.OUT:] + nrm[2 * M.IN:2 * M.IN + M.OUT]
    assert np.abs(y - y_ref).max() < 2e-2 * (np.abs(y_ref).max() + 1e-3)


def check_descriptors(engine_mod, b, seed):
    # thermal jitter: exact lattice distances (4 nm multiples) would sit on the
    # 20 nm cutoff, where FP32 and FP64 may decide differently
    coords = b.coords.copy()
    coords[:, :3] += np.random.default_rng(seed).normal(0.0, 0.01, size=(len(coords), 3)).astype(np.float32)
    e = engine_mod.Engine(b)
    e.upload_state(coords)
    X, _ = e.tea_training_data(targets=False)
    state = e.download_state()
    e.close()
    ref = M.descriptors(state, b.offsets, b.extra)
    assert np.all(X[b.extra != 0] == 0)
    # per feature column, relative to its norm (FP32 sums of up to a few hundred terms)
    for k in range(M.IN):
        den = np.linalg.norm(ref[:, k]) + 1e-12
        assert np.linalg.norm(X[:, k] - ref[:, k]) / den < 2e-5, (k, np.linalg.norm(X[:, k] - ref[:, k]) / den)


def test_descriptors_match_cpu_oracle(engine_mod):
    check_descriptors(engine_mod, small_system(seed=35, ntr=3, n_mon=20, n_free=200, tea=True, extra=2), 35)


def test_descriptors_match_cpu_oracle_ragged(engine_mod):
    p = synth.default_params(seed=36, hdi_on=1)
    check_descriptors(engine_mod, synth.ragged_batch(p, 5, seed=36, pf_range=(8, 20), free_range=(0, 300),
                                                     cube=60.0), 36)


def tea_dataset(engine_mod, seed, snapshots=12, every=5):
    b = small_system(seed=seed, ntr=4, n_mon=20, n_free=200, tea=True, tea_epsilon_freq=5, extra=0)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    Xs, Ts = [], []
    for k in range(snapshots):
        e.step(k * every, every)
        X, T = e.tea_training_data()
        Xs.append(X)
        Ts.append(T)
    e.close()
    return np.concatenate(Xs), np.concatenate(Ts)


def test_training_reduces_loss_and_beats_the_mean_predictor(engine_mod):
    X, T = tea_dataset(engine_mod, seed=31)
    Xv, Tv = tea_dataset(engine_mod, seed=32, snapshots=2)
    s = engine_mod.Surrogate(seed=7)
    losses = s.train(X, T, epochs=40, batch=512, lr=2e-3, seed=1)
    assert losses[-1] < 0.5 * losses[0], losses
    pred = s.predict(Xv)
    mse_net = ((pred[:, :3] - Tv[:, :3]) ** 2).mean()
    mse_mean = ((T[:, :3].mean(0) - Tv[:, :3]) ** 2).mean()       # the method without the network
    assert mse_net < 0.5 * mse_mean, (mse_net, mse_mean)


def test_training_is_deterministic(engine_mod):
    """Same data, seeds and batch: the same weights, bit for bit (every
    gradient reduction runs in a fixed order)."""
    rng = np.random.default_rng(9)
    X = rng.normal(2.0, 1.5, size=(3000, M.IN)).astype(np.float32)
    T = rng.normal(0.9, 0.05, size=(3000, M.OUT)).astype(np.float32)
    runs = []
    for _ in range(2):
        with engine_mod.Surrogate(seed=11) as s:
            losses = s.train(X, T, epochs=3, batch=512, lr=1e-3, seed=2)
            runs.append((losses, s.params()[0]))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])


def test_fallback_at_first_recheck_reproduces_exact_tea(engine_mod):
    """With max_err = 0 the first re-check (step 0) falls back and replaces the
    network's C_i and beta by the exact ones at once: the run is then the
    exact-TEA run, bit for bit."""
    b = small_system(seed=33, tea=True, tea_epsilon_freq=5)
    s = engine_mod.Surrogate(seed=8)
    e1 = engine_mod.Engine(b)
    e1.upload_state(b.coords)
    e1.set_surrogate(s, recheck_every=10, max_err=0.0)
    e1.step(0, 20)
    st = e1.surrogate_status()
    assert st["fell_back"] and st["rechecks"] == 1
    e2 = engine_mod.Engine(b)
    e2.upload_state(b.coords)
    e2.step(0, 20)
    assert np.array_equal(e1.download_state(), e2.download_state())
    assert np.array_equal(e1.download_rng(), e2.download_rng())


def test_learned_mode_runs_and_rechecks(engine_mod):
    X, T = tea_dataset(engine_mod, seed=34)
    s = engine_mod.Surrogate(seed=9)
    s.train(X, T, epochs=40, batch=512, lr=2e-3, seed=2)
    b = small_system(seed=34, ntr=4, n_mon=20, n_free=200, tea=True, tea_epsilon_freq=5, extra=0)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.set_surrogate(s, recheck_every=10, max_err=1.0)
    e.step(0, 30)
    st = e.surrogate_status()
    assert not st["fell_back"] and st["rechecks"] == 3
    assert np.isfinite(st["last_error"]) and st["last_error"] < 0.05, st
    assert np.all(np.isfinite(e.download_state()))
