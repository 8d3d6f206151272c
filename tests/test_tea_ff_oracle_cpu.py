"""The FP64 restatement of the learned mode's far field (oracle/tea_ff_oracle.py)
on the CPU: its tree restatement covers every ordered bead pair exactly once,
with everything near it equals the exact all-pairs product, and with the
workload's admissibility its approximation error stays small; the GPU tests
compare the kernels with it on the engine's own tree."""
import numpy as np

from oracle import tea_ff_oracle as O


def system(n=700, seed=0):
    rng = np.random.default_rng(seed)
    # a rod of lattice-like beads plus a cloud of free ones
    k = n // 2
    t = np.arange(k)
    rod = np.stack([12 * np.cos(2 * np.pi * (t % 13) / 13), 12 * np.sin(2 * np.pi * (t % 13) / 13),
                    4.0 * (t // 13)], 1)
    cloud = rng.uniform(-60, 60, size=(n - k, 3)) + np.array([0, 0, 60.0])
    x = np.concatenate([rod, cloud])
    F = rng.normal(size=(n, 3))
    R = rng.normal(size=(n, 3))
    ci = rng.uniform(0.05, 0.2, size=(n, 3))
    beta = np.full(n, 0.3)
    return x, F, R, ci, beta


def covered(layout, n):
    leaf_start, leaf_bead, near_start, near, node_range, node_parent, far_start, far = layout
    cov = np.zeros((n, n), np.int64)
    nleaf = len(leaf_start) - 1
    for L in range(nleaf):
        ti = leaf_bead[leaf_start[L]:leaf_start[L + 1]]
        for J in near[near_start[L]:near_start[L + 1]]:
            cov[np.ix_(ti, leaf_bead[leaf_start[J]:leaf_start[J + 1]])] += 1
    for N in range(len(node_parent)):
        ti = leaf_bead[node_range[2 * N]:node_range[2 * N + 1]]
        for J in far[far_start[N]:far_start[N + 1]]:
            cov[np.ix_(ti, leaf_bead[node_range[2 * J]:node_range[2 * J + 1]])] += 1
    np.fill_diagonal(cov, 1)
    return cov


def test_tree_covers_every_pair_once():
    x, *_ = system(2000)
    lay = O.tree_layout(x, np.arange(len(x)), 2.0, 0.85)
    assert np.all(covered(lay, len(x)) == 1)
    leaf_start, _, _, _, node_range, node_parent, far_start, _ = lay
    assert np.all(np.diff(leaf_start) <= 32)
    assert len(far_start) - 1 > len(leaf_start) - 1           # internal nodes take part
    assert (far_start[1:] > far_start[:-1])[len(leaf_start) - 1:].any()


def test_all_near_equals_exact():
    x, F, R, ci, beta = system(300)
    lay = O.tree_layout(x, np.arange(len(x)), 2.0, 1e-6)       # nothing is far
    assert len(lay[7]) == 0
    ff = O.effective_forces(x, F, R, ci, beta, 2.0, lay)
    ex = O.exact_effective_forces(x, F, R, ci, beta, 2.0, np.arange(len(x)))
    assert np.abs(ff - ex).max() <= 1e-10 * np.abs(ex).max()


def test_far_field_error_is_small():
    x, F, R, ci, beta = system()
    ex = O.exact_effective_forces(x, F, R, ci, beta, 2.0, np.arange(len(x)))
    errs = []
    for theta in (0.5, 0.85):
        lay = O.tree_layout(x, np.arange(len(x)), 2.0, theta)
        ff = O.effective_forces(x, F, R, ci, beta, 2.0, lay)
        d = ff - ex
        errs.append(np.sqrt((d ** 2).sum(1).mean() / (ex ** 2).sum(1).mean()))
    assert errs[1] < 0.03, errs
    assert errs[0] <= errs[1], errs
