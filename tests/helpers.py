"""Shared helpers of the test suite: systems, comparisons, cutoff margins."""
import math

import numpy as np

from mt_gb300 import synth

def lateral_sites():
    c, s = math.cos(2 * math.pi / 13), math.sin(2 * math.pi / 13)
    p1 = np.array([0.5 * 8.12 * (c - 1), 0.5 * 8.12 * s, -3 * 2.0 / 13])
    p2 = np.array([p1[0], -p1[1], -p1[2]])
    return p1, p2


def rotations(coords):
    """R = Rz(psi) Ry(theta) Rx(fi) per bead, float64 [n, 3, 3]."""
    fi, th, ps = (coords[:, 3].astype(np.float64), coords[:, 4].astype(np.float64), coords[:, 5].astype(np.float64))
    sf, cf, st, ct, sp, cp = np.sin(fi), np.cos(fi), np.sin(th), np.cos(th), np.sin(ps), np.cos(ps)
    R = np.empty((len(fi), 3, 3))
    R[:, 0, 0] = cp * ct
    R[:, 0, 1] = cp * st * sf - sp * cf
    R[:, 0, 2] = cp * st * cf + sp * sf
    R[:, 1, 0] = sp * ct
    R[:, 1, 1] = sp * st * sf + cp * cf
    R[:, 1, 2] = sp * st * cf - cp * sf
    R[:, 2, 0] = -st
    R[:, 2, 1] = ct * sf
    R[:, 2, 2] = ct * cf
    return R


def cutoff_margin(batch, coords):
    """Smallest distance (float64) of any list decision to its cutoff: LJ
    centre distance vs ljpairscutoff, site distances vs 2.5 nm.  List
    comparisons between two FP32 implementations are exact when this exceeds
    the FP32 rounding of the inputs."""
    p = batch.params
    p1, p2 = lateral_sites()
    worst = np.inf
    for t in range(batch.ntraj):
        b0, b1 = int(batch.offsets[t]), int(batch.offsets[t + 1])
        if b1 - b0 < 2:
            continue
        x = coords[b0:b1, :3].astype(np.float64)
        R = rotations(coords[b0:b1])
        uz = R[:, :, 2]
        cd = np.linalg.norm(x[:, None, :] - x[None, :, :], axis=-1)
        np.fill_diagonal(cd, np.inf)
        worst = min(worst, np.min(np.abs(cd - p.ljpairscutoff)))
        if p.is_assembly:
            h0 = batch.harmonic[batch.max_h * b0:batch.max_h * b1:batch.max_h]
            rmon = np.where(h0 < 0, -2.0, 2.0)
            si = x + rmon[:, None] * uz                            # site of i
            sj = x[None, :, :] - rmon[:, None, None] * uz[None, :, :]  # site of j as seen from i
            d = np.linalg.norm(sj - si[:, None, :], axis=-1)
            np.fill_diagonal(d, np.inf)
            worst = min(worst, np.min(np.abs(d - 2.5)))
            l1 = x + np.einsum("nij,j->ni", R, p1)
            l2 = x + np.einsum("nij,j->ni", R, p2)
            for a, c in ((l1, l2), (l2, l1)):
                d = np.linalg.norm(c[None, :, :] - a[:, None, :], axis=-1)
                np.fill_diagonal(d, np.inf)
                worst = min(worst, np.min(np.abs(d - 2.5)))
    return worst


def rel_norm(a, b):
    """||a - b|| / ||b|| over all entries (b the reference), with a floor."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def small_system(seed=1, ntr=2, n_mon=12, n_free=40, tea=False, extra=2, **over):
    p = synth.default_params(seed=seed, hdi_on=int(tea), **over)
    b = synth.uniform_batch(p, ntr, n_mon, n_free, seed=seed, radius=8.12, psi_mode="make_mt", cube=40.0,
                            thermal=0.05, n_extra_dimers=extra)
    return b


def system_with_margin(seed=1, min_margin=2e-4, **kw):
    """small_system re-drawn until no list decision sits within min_margin nm of its cutoff."""
    for s in range(seed, seed + 50):
        b = small_system(seed=s, **kw)
        if cutoff_margin(b, b.coords) > min_margin:
            return b
    raise RuntimeError("no system with the requested cutoff margin")


def golden_batch(d):
    """Rebuilds a Batch from a golden .npz."""
    from mt_gb300._abi import MtgParams
    p = MtgParams()
    for k in d.files:
        if k.startswith("param_"):
            setattr(p, k[6:], d[k].item())
    off = d["offsets"]
    b = synth.Batch(params=p, offsets=off, coords=d["coords"], mon_type=d["mon_type"], fixed=d["fixed"],
                    extra=d["extra"], gtp=d["gtp"], on_tubule=d["on_tubule"], harmonic_count=d["harmonic_count"],
                    harmonic=d["harmonic"], zs=d["zs"])
    sizes = np.diff(off)
    if len(set(sizes.tolist())) == 1:
        b.uniform_ntot = int(sizes[0])
    return b


def with_lone_monomers(b, local=(160, 161)):
    """Turns the free dimer at the given local indices of every trajectory into
    two monomers without a harmonic partner: count 0 and entry -1, as
    read_PDB leaves such a bead (src/preparator.cpp:340); pairs_kernel then
    takes R_MON = -r_mon and skips j = 1 for it (src/compute_cuda.cu:548,565,599)."""
    for t in range(b.ntraj):
        for i in local:
            g = int(b.offsets[t]) + i
            b.harmonic_count[g] = 0
            b.harmonic[g * b.max_h:(g + 1) * b.max_h] = -1
    return b


def per_bead_rel(got, ref, active, floor_frac):
    """Largest per-bead relative error of vector rows: |got_i - ref_i| /
    max(|ref_i|, floor_frac * RMS_i |ref_i|) over the active beads (row norms;
    the floor keeps beads whose value nearly cancels from dominating)."""
    got = np.asarray(got, np.float64)[active]
    ref = np.asarray(ref, np.float64)[active]
    if got.ndim == 1:
        got, ref = got[:, None], ref[:, None]
    mag = np.linalg.norm(ref, axis=1)
    rms = float(np.sqrt(np.mean(mag ** 2))) if len(mag) else 0.0
    if rms == 0.0:
        return float(np.max(np.linalg.norm(got - ref, axis=1), initial=0.0)), 0.0
    d = np.linalg.norm(got - ref, axis=1)
    return float(np.max(d / np.maximum(mag, floor_frac * rms))), rms


def site_tie_distance(batch, coords, g):
    """FP64 distance of the closest longitudinal or lateral site test of bead g
    (global index) to the 2.5 nm cutoff, over the beads of its trajectory."""
    t = int(np.searchsorted(batch.offsets, g, side="right") - 1)
    b0, b1 = int(batch.offsets[t]), int(batch.offsets[t + 1])
    x = coords[b0:b1, :3].astype(np.float64)
    R = rotations(coords[b0:b1])
    uz = R[:, :, 2]
    i = g - b0
    p1, p2 = lateral_sites()
    h0 = batch.harmonic[batch.max_h * g]
    rmon = -2.0 if h0 < 0 else 2.0
    worst = np.inf
    si = x[i] + rmon * uz[i]
    sj = x - rmon * uz
    d = np.linalg.norm(sj - si, axis=1)
    d[i] = np.inf
    worst = min(worst, float(np.min(np.abs(d - 2.5))))
    l1 = x + np.einsum("nij,j->ni", R, p1)
    l2 = x + np.einsum("nij,j->ni", R, p2)
    for a, c in ((l1, l2), (l2, l1)):
        d = np.linalg.norm(c - a[i], axis=1)
        d[i] = np.inf
        worst = min(worst, float(np.min(np.abs(d - 2.5))))
    return worst


def ulp32(x):
    """Spacing of FP32 numbers at |x|."""
    return np.spacing(np.abs(np.asarray(x, np.float32))).astype(np.float64)
