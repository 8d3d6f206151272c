"""CPU oracle of the TEA surrogate network (TEST INFRASTRUCTURE ONLY).

A numpy restatement of the 32-128-128-128-4 SiLU perceptron and its MSE
loss, with the parameter layout of include/mtg.h (mtg_surrogate_get_params):
forward, analytic backward in FP64, optionally emulating the GPU's BF16
rounding of weights, inputs and activations so that the comparison isolates
the kernels' accumulation order.
"""
import numpy as np

IN, HID, OUT = 32, 128, 4
OFF_W1 = 0
OFF_W2 = OFF_W1 + HID * IN
OFF_W3 = OFF_W2 + HID * HID
OFF_W4 = OFF_W3 + HID * HID
OFF_B = OFF_W4 + OUT * HID
NPARAMS = OFF_B + 3 * HID + OUT


def bf16(x):
    """Round to bfloat16 (nearest even) and back, elementwise."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    W1 = p[OFF_W1:OFF_W2].reshape(HID, IN)
    W2 = p[OFF_W2:OFF_W3].reshape(HID, HID)
    W3 = p[OFF_W3:OFF_W4].reshape(HID, HID)
    W4 = p[OFF_W4:OFF_B].reshape(OUT, HID)
    b = p[OFF_B:]
    return [W1, W2, W3, W4], [b[:HID], b[HID:2 * HID], b[2 * HID:3 * HID], b[3 * HID:]]


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, Xn, emulate_bf16=False):
    """Xn: normalised inputs [n, 32].  Returns (y [n, 4], cache)."""
    W, b = unpack(p)
    r = bf16 if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    h = r(Xn)
    zs, hs = [], [h]
    for l in range(3):
        z = h @ r(W[l]).T + b[l]
        zs.append(z)
        h = r(silu(z))
        hs.append(h)
    y = h @ r(W[3]).T + b[3]
    return y, (zs, hs)


def loss_grad(p, Xn, Tn, emulate_bf16=False):
    """MSE loss (mean over samples and outputs) and its gradient in the parameter layout."""
    W, b = unpack(p)
    r = bf16 if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    y, (zs, hs) = forward(p, Xn, emulate_bf16)
    n = len(Xn)
    e = y - Tn
    loss = float(np.mean(e * e))
    d = r(2.0 * e / (n * OUT))
    g = np.zeros(NPARAMS)
    gW = [None] * 4
    gb = [None] * 4
    for l in range(3, -1, -1):
        gW[l] = d.T @ hs[l]
        gb[l] = d.sum(0)
        if l > 0:
            dh = d @ r(W[l])
            d = r(dh * dsilu(zs[l - 1]))
    g[OFF_W1:OFF_W2] = gW[0].ravel()
    g[OFF_W2:OFF_W3] = gW[1].ravel()
    g[OFF_W3:OFF_W4] = gW[2].ravel()
    g[OFF_W4:OFF_B] = gW[3].ravel()
    g[OFF_B:OFF_B + HID] = gb[0]
    g[OFF_B + HID:OFF_B + 2 * HID] = gb[1]
    g[OFF_B + 2 * HID:OFF_B + 3 * HID] = gb[2]
    g[OFF_B + 3 * HID:] = gb[3]
    return loss, g


def normalise(X, T, norm):
    """Applies the 72-float normalisation of mtg_surrogate_get_params."""
    xm, xis, tm, ts = norm[:IN], norm[IN:2 * IN], norm[2 * IN:2 * IN + OUT], norm[2 * IN + OUT:]
    return (np.asarray(X, np.float64) - xm) * xis, (np.asarray(T, np.float64) - tm) / ts


DESC_CUT = 20.0
SHELLS = (0.0, 5.0, 10.0, 20.0)


def descriptors(coords, offsets, extra):
    """The 32-feature per-bead descriptor in FP64 (no reference counterpart:
    the learned TEA's input).  For each bead i of trajectory t, over the
    non-extra beads j != i of t with 0 < r_ij < 20 nm, in the shells
    [0,5), [5,10), [10,20) nm: count, sum 1/r, 1/r^2, 1/r^3, and
    sum u_a u_b / r for (a,b) = xx, yy, zz, xy, xz, yz with u = (r_j - r_i)/r;
    then log N' (non-extra beads of t) and |r_i - centroid of t| / 100 nm.
    Extra beads get all zeros."""
    pos = np.asarray(coords, np.float64)[:, :3]
    extra = np.asarray(extra).astype(bool)
    out = np.zeros((len(pos), IN))
    for t in range(len(offsets) - 1):
        a, b = int(offsets[t]), int(offsets[t + 1])
        p = pos[a:b]
        act = ~extra[a:b]
        n_act = int(act.sum())
        cen = p[act].mean(0) if n_act else np.zeros(3)
        d = p[None, :, :] - p[:, None, :]            # d[i, j] = r_j - r_i
        r = np.sqrt((d * d).sum(-1))
        ok = act[None, :] & (r > 0) & (r < DESC_CUT)
        np.fill_diagonal(ok, False)
        with np.errstate(divide="ignore", invalid="ignore"):
            ri = np.where(ok, 1.0 / r, 0.0)
            u = np.where(ok[..., None], d * ri[..., None], 0.0)
        terms = [np.ones_like(ri), ri, ri ** 2, ri ** 3,
                 u[..., 0] ** 2 * ri, u[..., 1] ** 2 * ri, u[..., 2] ** 2 * ri,
                 u[..., 0] * u[..., 1] * ri, u[..., 0] * u[..., 2] * ri, u[..., 1] * u[..., 2] * ri]
        for s in range(3):
            m = ok & (r >= SHELLS[s]) & (r < SHELLS[s + 1])
            for k, v in enumerate(terms):
                out[a:b, 10 * s + k] = np.where(m, v, 0.0).sum(1)
        out[a:b, 30] = np.log(max(n_act, 1))
        out[a:b, 31] = np.sqrt(((p - cen) ** 2).sum(1)) * 0.01
        out[a:b][~act] = 0.0
    return out
