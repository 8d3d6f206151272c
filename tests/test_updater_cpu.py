"""The vectorised hydrolysis restatement agrees with the loop restatement of
src/updater.cpp:229-257 (CPU only)."""
import numpy as np

from oracle import updater_oracle as U


def test_hydrolyse_vec_matches_loop():
    rng = np.random.default_rng(3)
    offsets = np.array([0, 40, 71, 120, 122])
    nb = offsets[-1]
    gtp = rng.integers(0, 2, nb)
    extra = rng.integers(0, 2, nb) * (rng.uniform(size=nb) < 0.2)
    cur = rng.integers(0, 2, nb)
    prev = rng.integers(0, 2, nb)
    probs = rng.uniform(0, 0.05, size=1000)
    it = iter(probs)
    ref, n_ref, _ = U.hydrolyse(offsets, gtp, extra, cur, prev, lambda: next(it))
    got, n = U.hydrolyse_vec(offsets, gtp, extra, cur, prev, lambda m: probs[:m])
    assert n == n_ref and np.array_equal(got, ref)
