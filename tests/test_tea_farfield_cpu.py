"""Why a local surrogate cannot replace the TEA mobility product at 1%:
the RPY coupling decays as 1/r while the number of beads at distance r
grows as r^2, so the far field carries much of the correlated displacement.
Truncating sum_j T_ij g_j (src/bdhitea_kernel.cu:104-213) at a cutoff, on a
seeded lattice + free-tubulin trajectory, leaves an RMS mobility error above 1% even
at 30 nm (FP64, CPU only; the full-size study is quoted in the design notes)."""
import numpy as np

from mt_gb300 import synth


def rpy_blocks(x, a=2.0):
    d = x[None, :, :] - x[:, None, :]
    r = np.linalg.norm(d, axis=-1)
    ra = r / a
    u = d / np.maximum(r, 1e-12)[..., None]
    ira = 1.0 / np.maximum(ra, 1e-12)
    far = ra > 2
    crr = np.where(far, 0.75 * ira * (1 - 2 * ira ** 2), 3 * ra / 32)
    cii = np.where(far, 0.75 * ira * (1 + 2 / 3 * ira ** 2), 1 - 9 * ra / 32)
    np.fill_diagonal(cii, 0.0)
    np.fill_diagonal(crr, 0.0)
    return cii, crr, u, r


def mobility_error_of_cutoff(n_mon, n_free, cube, cutoffs, seed=3):
    t = synth.make_trajectory(n_mon, n_free, seed=seed, cube=cube)
    x = t.coords[:, :3].astype(np.float64)
    n = len(x)
    cii, crr, u, r = rpy_blocks(x)
    # TEA epsilon, beta and C_i (src/bdhitea_kernel.cu:61-101, src/bdhitea.cu:75-116)
    ci = (cii ** 2)[..., None] + ((2 * cii + crr) * crr)[..., None] * u ** 2
    ci = ci.sum(1)
    eps_i = (3 * cii + crr * u.sum(-1) ** 2).sum(1)
    e = eps_i.sum() / (3 * n * (3 * n - 3))
    a_ = (3 * n - 1) * e * e - (3 * n - 2) * e
    beta = (1 - np.sqrt(1 - a_)) / a_
    C = 1 / np.sqrt(1 + beta ** 2 * ci)
    rng = np.random.default_rng(0)
    R = rng.normal(size=(n, 3))
    F = rng.normal(size=(n, 3)) * 0.1

    def disp(mask):
        g = F[None, :, :] + beta * C[:, None, :] * R[None, :, :]
        ug = (u * g).sum(-1)
        Tg = ((cii * mask)[..., None] * g + (crr * mask * ug)[..., None] * u).sum(1)
        return F + C * R + Tg

    ex = disp(np.ones((n, n)))
    return {rc: float(np.sqrt(((disp((r < rc).astype(float)) - ex) ** 2).sum(1).mean() / (ex ** 2).sum(1).mean()))
            for rc in cutoffs}


def test_truncated_mobility_misses_one_percent():
    err = mobility_error_of_cutoff(40, 600, 60.0, (10.0, 20.0, 30.0))
    assert err[10.0] > err[20.0] > err[30.0]
    assert err[30.0] > 0.01, err
