"""The bounded waits of the tensor-core kernels end in an error status, not
a hang: with the surrogate's wait limit at 0 polls, every wait of the
inference for a layer's MMAs gives up at once, the kernel records the
timeout, lets the MMAs it issued finish (a second wait at the full default
limit), frees its tensor memory and returns; the call reports MTG_E_TIMEOUT
and the context stays usable.  The next call with the default limit runs
normally and matches the oracle, through mtg_surrogate_predict and through
the learned mode of the step loop.  (The reference has no bounded wait: a
CUDA error ends its program, src/Cuda.h:120-135.)"""
import numpy as np
import pytest

from helpers import small_system

pytestmark = pytest.mark.gpu


def test_inference_timeout_reported_then_recovers(engine_mod):
    from mt_gb300 import _abi
    from oracle import mlp_oracle as M
    X = np.random.default_rng(7).normal(size=(300, M.IN)).astype(np.float32)
    with engine_mod.Surrogate(seed=21) as s:
        rc, y0 = s.predict_raw(X)
        assert rc == 0
        s.set_wait_limit(0)
        rc, _ = s.predict_raw(X)
        assert rc == _abi.MTG_E_TIMEOUT, rc
        assert b"bounded wait" in engine_mod.load().mtg_last_error_string()
        s.set_wait_limit(-1)
        rc, y1 = s.predict_raw(X)
        assert rc == 0 and np.array_equal(y0, y1)
        prm, nrm = s.params()
    Xn, _ = M.normalise(X, np.zeros((len(X), M.OUT)), nrm)
    y_ref, _ = M.forward(prm, Xn, emulate_bf16=True)
    y_ref = y_ref * nrm[2 * M.IN + M.OUT:] + nrm[2 * M.IN:2 * M.IN + M.OUT]
    assert float(np.abs(y1 - y_ref).max() / (np.abs(y_ref).max() + 1e-3)) < 2e-2


def test_learned_step_timeout_reported_then_recovers(engine_mod):
    from mt_gb300 import _abi
    b = small_system(seed=22, tea=True, tea_epsilon_freq=5)
    s = engine_mod.Surrogate(seed=22)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    s.set_wait_limit(0)
    e.set_surrogate(s, recheck_every=10, max_err=1.0)
    assert e.step_raw(0, 5) == _abi.MTG_E_TIMEOUT
    # the same engine and surrogate, default limit: steps run and the noise
    # streams advance exactly as in an engine that never timed out
    s.set_wait_limit(-1)
    e.set_surrogate(s, recheck_every=10, max_err=1.0)    # new graphs with the default limit
    e.upload_state(b.coords)
    rng0 = e.download_rng()
    e.step(5, 10)
    assert np.all(np.isfinite(e.download_state()))
    e2 = engine_mod.Engine(b)
    e2.upload_state(b.coords)
    e2.upload_rng(rng0)
    e2.rebuild_pairs()                                   # e holds the lists of step 0 of the same state
    e2.set_surrogate(s, recheck_every=10, max_err=1.0)
    e2.step(5, 10)
    assert np.array_equal(e.download_state(), e2.download_state())
    e.close()
    e2.close()
    s.close()
