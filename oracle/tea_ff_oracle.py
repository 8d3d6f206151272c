"""FP64 restatement of the far-field approximation of the learned TEA
mobility product (TEST INFRASTRUCTURE ONLY: the checker of the CUDA kernels
k_ff_p2m / k_ff_m2l / k_ff_step, never a product path).

Given the engine's grouping of beads into leaves with near and far source
leaves (mtg_tea_farfield_layout), the positions x, forces F, random forces R,
row sums ci and beta per bead, it evaluates

    f_i = F_i + C_i o R_i + sum_{j in near leaves, j != i} T_ij (F_j + beta C_i o R_j)
          + sum_n w_n(x_i) (A_n + sum_k beta C_ik B_kn)

with C_i = 1 / sqrt(1 + beta^2 ci_i) (integrateTea_force,
src/bdhitea_kernel.cu:104-213), T the RPY tensor in units of the bead's own
mobility with both branches (src/bdhitea_kernel.cu:38-58), and for every far
leaf J of the target leaf I: proxies y_m of J (the 8 nodes c +- h/sqrt(2) of
its bounding box), charges Q_m = sum_{j in J} w_m(x_j) (F_j, R_j) with the
trilinear Lagrange weights w of those nodes, target proxies x_n of I, and
A_n = sum T(y_m - x_n) QF_m, B_kn = sum T(y_m - x_n) e_k QR_mk.
"""
import numpy as np

S = 1.0 / np.sqrt(2.0)


def rpy(d, a):
    """cii, crr (both branches) and unit vectors of separations d [..., 3]."""
    r = np.linalg.norm(d, axis=-1)
    ra = r / a
    with np.errstate(divide="ignore", invalid="ignore"):
        u = d / r[..., None]
        cii = np.where(ra > 2, 0.75 / ra * (1 + 2 / (3 * ra ** 2)), 1 - 9 * ra / 32)
        crr = np.where(ra > 2, 0.75 / ra * (1 - 2 / ra ** 2), 3 * ra / 32)
    return cii, crr, u


def box(x):
    lo, hi = x.min(0), x.max(0)
    return (lo + hi) / 2, np.maximum((hi - lo) / 2, 1e-3)


def weights(x, c, h):
    t = (x - c) / (h * S)
    l = np.stack([0.5 * (1 - t), 0.5 * (1 + t)], axis=-1)        # [n, 3, 2]
    m = np.arange(8)
    return l[:, 0, m & 1] * l[:, 1, (m >> 1) & 1] * l[:, 2, (m >> 2) & 1]


def proxies(c, h):
    m = np.arange(8)
    sg = np.stack([np.where(m & 1, 1.0, -1.0), np.where(m & 2, 1.0, -1.0), np.where(m & 4, 1.0, -1.0)], axis=1)
    return c + sg * S * h


def effective_forces(x, F, R, ci, beta, a, layout):
    """f_i as above, [n, 3] FP64, for the beads of the leaves (others zero)."""
    leaf_start, leaf_bead, near_start, near, far_start, far = layout
    x, F, R, ci = (np.asarray(v, np.float64)[:, :3] for v in (x, F, R, ci))
    beta = np.asarray(beta, np.float64)
    nl = len(leaf_start) - 1
    idx = [leaf_bead[leaf_start[L]:leaf_start[L + 1]] for L in range(nl)]
    W, Y, QF, QR = [], [], [], []
    for L in range(nl):
        c, h = box(x[idx[L]])
        w = weights(x[idx[L]], c, h)
        W.append(w)
        Y.append(proxies(c, h))
        QF.append(w.T @ F[idx[L]])
        QR.append(w.T @ R[idx[L]])
    out = np.zeros_like(x)
    for I in range(nl):
        ti = idx[I]
        C = 1 / np.sqrt(1 + beta[ti, None] ** 2 * ci[ti])          # [nI, 3]
        cb = beta[ti, None] * C
        src = np.concatenate([idx[J] for J in near[near_start[I]:near_start[I + 1]]])
        d = x[src][None, :, :] - x[ti][:, None, :]
        cii, crr, u = rpy(d, a)
        self_pair = src[None, :] == ti[:, None]
        cii = np.where(self_pair, 0.0, cii)
        crr = np.where(self_pair, 0.0, crr)
        u = np.where(self_pair[..., None], 0.0, u)
        g = F[src][None, :, :] + cb[:, None, :] * R[src][None, :, :]
        near_sum = (cii[..., None] * g + (crr * (u * g).sum(-1))[..., None] * u).sum(1)
        A = np.zeros((8, 3))
        Bk = np.zeros((3, 8, 3))
        for J in far[far_start[I]:far_start[I + 1]]:
            dd = Y[J][None, :, :] - Y[I][:, None, :]                # [n, m, 3]
            cii_f, crr_f, uf = rpy(dd, a)
            A += (cii_f[..., None] * QF[J][None] + (crr_f * (uf * QF[J][None]).sum(-1))[..., None] * uf).sum(1)
            for k in range(3):
                qk = QR[J][:, k]                                     # [m]
                Bk[k] += (crr_f * uf[..., k] * qk[None])[..., None].__mul__(uf).sum(1)
                Bk[k][:, k] += (cii_f * qk[None]).sum(1)
        far_sum = W[I] @ A + sum(cb[:, k:k + 1] * (W[I] @ Bk[k]) for k in range(3))
        out[ti] = F[ti] + C * R[ti] + near_sum + far_sum
    return out


def exact_effective_forces(x, F, R, ci, beta, a, beads):
    """f_i with every pair of the trajectory summed exactly, for the given beads
    (all of one trajectory, non-extra)."""
    x, F, R, ci = (np.asarray(v, np.float64)[:, :3] for v in (x, F, R, ci))
    beta = np.asarray(beta, np.float64)
    out = np.zeros_like(x)
    for s in range(0, len(beads), 256):
        ti = beads[s:s + 256]
        C = 1 / np.sqrt(1 + beta[ti, None] ** 2 * ci[ti])
        cb = beta[ti, None] * C
        d = x[beads][None, :, :] - x[ti][:, None, :]
        cii, crr, u = rpy(d, a)
        self_pair = beads[None, :] == ti[:, None]
        cii = np.where(self_pair, 0.0, cii)
        crr = np.where(self_pair, 0.0, crr)
        u = np.where(self_pair[..., None], 0.0, u)
        g = F[beads][None, :, :] + cb[:, None, :] * R[beads][None, :, :]
        out[ti] = F[ti] + C * R[ti] + (cii[..., None] * g + (crr * (u * g).sum(-1))[..., None] * u).sum(1)
    return out
