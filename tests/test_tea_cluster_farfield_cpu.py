"""A particle-cluster far field for the TEA mobility product (FP64, CPU
only): the exact sum_j T_ij g_j (src/bdhitea_kernel.cu:104-213) against
near pairs summed exactly plus far clusters (k-d tree leaves of 32 beads)
expanded to monopole + dipole + quadrupole when their centres are farther
apart than (R_I + R_J) / theta.  The error falls with theta and with the
expansion order; the cost (near pairs and cluster evaluations per bead) is
what bounds the speed-up of such a scheme.  The full-size study (one
5600-bead trajectory) is quoted in the design notes."""
import numpy as np

from mt_gb300 import synth

A = 2.0


def t_apply(d, g):
    """Far-field RPY tensor (units of the bead's own mobility) applied to g."""
    r = np.linalg.norm(d, axis=-1)
    cii = 0.75 * A * (1 / r + 2 * A * A / (3 * r ** 3))
    crr = 0.75 * A * (1 / r ** 3 - 2 * A * A / r ** 5)
    return cii[..., None] * g + (crr * (d * g).sum(-1))[..., None] * d


def pair_sum(x, g, i, idx):
    """Exact sum over j in idx (j != i), both RPY branches."""
    idx = idx[idx != i]
    d = x[idx] - x[i]
    r = np.linalg.norm(d, axis=1)
    ra = r / A
    u = d / r[:, None]
    cii = np.where(ra > 2, 0.75 / ra * (1 + 2 / (3 * ra ** 2)), 1 - 9 * ra / 32)
    crr = np.where(ra > 2, 0.75 / ra * (1 - 2 / ra ** 2), 3 * ra / 32)
    return (cii[:, None] * g[idx] + (crr * (u * g[idx]).sum(1))[:, None] * u).sum(0)


def leaves(x, idx, size):
    if len(idx) <= size:
        return [idx]
    p = x[idx]
    o = idx[np.argsort(p[:, np.argmax(p.max(0) - p.min(0))], kind="stable")]
    h = len(o) // 2
    return leaves(x, o[:h], size) + leaves(x, o[h:], size)


def cluster_error(x, g, theta, order, size=32, h=1e-3):
    n = len(x)
    L = leaves(x, np.arange(n), size)
    cen = np.array([x[l].mean(0) for l in L])
    rad = np.array([np.linalg.norm(x[l] - c, axis=1).max() for l, c in zip(L, cen)])
    m0 = np.array([g[l].sum(0) for l in L])
    m1 = np.array([np.einsum("jk,jl->kl", x[l] - c, g[l]) for l, c in zip(L, cen)])
    m2 = np.array([np.einsum("jk,jm,jl->kml", x[l] - c, x[l] - c, g[l]) for l, c in zip(L, cen)])
    err2 = tot2 = 0.0
    near_pairs = far_evals = 0
    for I, li in enumerate(L):
        far = np.linalg.norm(cen - cen[I], axis=1) > (rad + rad[I]) / theta
        near = np.concatenate([L[J] for J in np.nonzero(~far)[0]])
        near_pairs += len(li) * len(near)
        far_evals += len(li) * int(far.sum())
        for i in li:
            exact = pair_sum(x, g, i, np.arange(n))
            approx = pair_sum(x, g, i, near)
            D = cen[far] - x[i]
            approx += t_apply(D, m0[far]).sum(0)
            e = np.eye(3) * h
            if order >= 1:
                for k in range(3):
                    approx += ((t_apply(D + e[k], m1[far][:, k]) - t_apply(D - e[k], m1[far][:, k])) / (2 * h)).sum(0)
            if order >= 2:
                for k in range(3):
                    for m in range(3):
                        G = m2[far][:, k, m]
                        d2 = (t_apply(D + e[k] + e[m], G) - t_apply(D + e[k] - e[m], G)
                              - t_apply(D - e[k] + e[m], G) + t_apply(D - e[k] - e[m], G)) / (4 * h * h)
                        approx += 0.5 * d2.sum(0)
            err2 += ((approx - exact) ** 2).sum()
            tot2 += ((exact + g[i]) ** 2).sum()
    return np.sqrt(err2 / tot2), near_pairs / n, far_evals / n


def test_cluster_far_field_error_and_cost():
    t = synth.make_trajectory(40, 600, seed=3, cube=60.0, thermal=0.05)
    x = t.coords[:, :3].astype(np.float64)
    g = np.random.default_rng(0).normal(size=(len(x), 3))
    res = {(th, o): cluster_error(x, g, th, o) for th in (0.5, 1.0) for o in (1, 2)}
    for o in (1, 2):
        assert res[(0.5, o)][0] < res[(1.0, o)][0]            # tighter acceptance, smaller error
        assert res[(0.5, o)][1] > res[(1.0, o)][1]            # ... and more direct pairs
    for th in (0.5, 1.0):
        assert res[(th, 2)][0] < res[(th, 1)][0]              # the quadrupole term helps
    assert res[(0.5, 2)][0] < 1e-3 and res[(1.0, 2)][0] > 2e-3
