"""FP64 restatement of the far-field approximation of the learned TEA
mobility product (TEST INFRASTRUCTURE ONLY: the checker of the CUDA kernels
k_ff_p2m / k_ff_m2l / k_ff_step, never a product path).

Given the engine's grouping (mtg_tea_farfield_layout): leaves of beads with
their near source leaves, and a tree of nodes over the leaves (nodes
0 .. nleaf-1 are the leaves, every node a contiguous range of the leaf bead
order) with, per target node, its far source nodes; and the positions x,
forces F, random forces R, row sums ci and beta per bead, it evaluates

    f_i = F_i + C_i o R_i + sum_{j in near leaves, j != i} T_ij (F_j + beta C_i o R_j)
          + sum_{nodes N containing i} sum_n w^N_n(x_i) (A^N_n + sum_k beta C_ik B^N_kn)

with C_i = 1 / sqrt(1 + beta^2 ci_i) (integrateTea_force,
src/bdhitea_kernel.cu:104-213), T the RPY tensor in units of the bead's own
mobility with both branches (src/bdhitea_kernel.cu:38-58), and for every far
node J of a target node N: proxies y_m of J (the 8 nodes c +- h/sqrt(2) of
its bounding box), charges Q_m = sum_{j in J} w_m(x_j) (F_j, R_j) with the
trilinear Lagrange weights w of those nodes, target proxies x_n of N, and
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
    leaf_start, leaf_bead, near_start, near, node_range, node_parent, far_start, far = layout
    x, F, R, ci = (np.asarray(v, np.float64)[:, :3] for v in (x, F, R, ci))
    beta = np.asarray(beta, np.float64)
    nl = len(leaf_start) - 1
    nn = len(node_parent)
    idx = [leaf_bead[node_range[2 * N]:node_range[2 * N + 1]] for N in range(nn)]
    boxes, Y, QF, QR = [], [], [], []
    for N in range(nn):
        c, h = box(x[idx[N]])
        w = weights(x[idx[N]], c, h)
        boxes.append((c, h))
        Y.append(proxies(c, h))
        QF.append(w.T @ F[idx[N]])
        QR.append(w.T @ R[idx[N]])
    # far potentials at every target node's proxies
    A = np.zeros((nn, 8, 3))
    Bk = np.zeros((nn, 3, 8, 3))
    for N in range(nn):
        for J in far[far_start[N]:far_start[N + 1]]:
            dd = Y[J][None, :, :] - Y[N][:, None, :]                # [n, m, 3]
            cii_f, crr_f, uf = rpy(dd, a)
            A[N] += (cii_f[..., None] * QF[J][None] + (crr_f * (uf * QF[J][None]).sum(-1))[..., None] * uf).sum(1)
            for k in range(3):
                qk = QR[J][:, k]                                     # [m]
                Bk[N, k] += ((crr_f * uf[..., k] * qk[None])[..., None] * uf).sum(1)
                Bk[N, k][:, k] += (cii_f * qk[None]).sum(1)
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
        acc = F[ti] + C * R[ti] + (cii[..., None] * g + (crr * (u * g).sum(-1))[..., None] * u).sum(1)
        N = I
        while N >= 0:      # the leaf and its ancestors
            if far_start[N + 1] > far_start[N]:
                w = weights(x[ti], *boxes[N])
                acc += w @ A[N] + sum(cb[:, k:k + 1] * (w @ Bk[N, k]) for k in range(3))
            N = node_parent[N]
        out[ti] = acc
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


NODE_THETA = 0.7     # theta factor for node pairs that involve an internal node
MARGIN = 1.0         # nm added to each radius in the far test


def tree_layout(x, beads, a, theta, leaf=32):
    """The engine's tree for one trajectory (the beads given, all non-extra),
    restated: k-d bisection on the longest extent (median rounded to a
    multiple of `leaf` while more than two leaves' worth remain, ties by
    index), then the dual traversal from (root, root) into near leaf pairs and
    far node pairs.  Returns the layout of effective_forces (global bead
    indices; leaves first, internal nodes after them by decreasing size)."""
    x = np.asarray(x, np.float64)[:, :3]
    nodes = []                                    # [beg, end, children, parent]
    order = np.array(beads, np.int64)

    def split(beg, end, parent):
        me = len(nodes)
        nodes.append([beg, end, None, parent])
        n = end - beg
        if n <= leaf:
            return me
        p = x[order[beg:end]]
        ax = int(np.argmax(p.max(0) - p.min(0)))
        k = max(leaf, (n // 2) // leaf * leaf) if n > 2 * leaf else n // 2
        seg = order[beg:end]
        order[beg:end] = seg[np.lexsort((seg, x[seg, ax]))]
        l = split(beg, beg + k, me)
        r = split(beg + k, end, me)
        nodes[me][2] = (l, r)
        return me

    split(0, len(order), -1)
    c, r = [], []
    for beg, end, _, _ in nodes:
        p = x[order[beg:end]]
        cc = (p.min(0) + p.max(0)) / 2
        c.append(cc)
        r.append(np.linalg.norm(p - cc, axis=1).max())
    near = {k: [] for k in range(len(nodes)) if nodes[k][2] is None}
    far = {}
    stack = [(0, 0)]
    while stack:
        I, J = stack.pop()
        leaves = nodes[I][2] is None and nodes[J][2] is None
        th = theta if leaves else theta * NODE_THETA
        d = np.linalg.norm(c[J] - c[I])
        if I != J and d * th > r[I] + r[J] + 2 * MARGIN and d - r[I] - r[J] > 4 * a + 2 * MARGIN:
            far.setdefault(I, []).append(J)
        elif leaves:
            near[I].append(J)
        elif nodes[J][2] is None or (nodes[I][2] is not None and r[I] >= r[J]):
            stack += [(nodes[I][2][1], J), (nodes[I][2][0], J)]
        else:
            stack += [(I, nodes[J][2][1]), (I, nodes[J][2][0])]
    leaf_ids = [k for k in range(len(nodes)) if nodes[k][2] is None]          # depth-first order
    inner = sorted((k for k in range(len(nodes)) if nodes[k][2] is not None),
                   key=lambda k: -(nodes[k][1] - nodes[k][0]))
    new = {k: i for i, k in enumerate(leaf_ids + inner)}
    nn = len(nodes)
    node_range = np.zeros(2 * nn, np.int64)
    node_parent = np.zeros(nn, np.int64)
    for k, (beg, end, _, par) in enumerate(nodes):
        node_range[2 * new[k]:2 * new[k] + 2] = beg, end
        node_parent[new[k]] = new[par] if par >= 0 else -1
    leaf_start = np.array([nodes[k][0] for k in leaf_ids] + [len(order)], np.int64)
    near_start, near_l = [0], []
    for k in leaf_ids:
        near_l += sorted(new[J] for J in near[k])
        near_start.append(len(near_l))
    far_start, far_l = [0], []
    for k in leaf_ids + inner:
        far_l += [new[J] for J in far.get(k, [])]
        far_start.append(len(far_l))
    return (leaf_start, order, np.array(near_start), np.array(near_l, np.int64), node_range, node_parent,
            np.array(far_start), np.array(far_l, np.int64))
