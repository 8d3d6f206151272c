"""Seeded synthetic microtubule systems.

The lattice follows the generator semantics of the reference's
scripts/make_mt.py:29-66: protofilament k (chain A..M) holds monomers m with
z = 4 m + (12/13) k nm, azimuth alpha_k = 2 pi k / 13, (x, y) = R (cos(-alpha_k),
sin(-alpha_k)); even m are alpha ("CA", type 0), odd m beta ("CB", type 1);
resid = m // 2 + 1, atom id = m + n_mon k + 1.  The reference sets psi =
-alpha_k; the benchmark workloads use the lattice radius and all-zero angles
they are specified with.  A plus-end tail (make_mt.py:36-40) tilts the last
monomers outwards by ``bend`` rad each.

Free tubulin is placed as dimers (CA + CB, harmonic partners), because the
reference assumes every bead has a harmonic partner (pairs_kernel reads
harmonic[max*i] unconditionally, src/compute_cuda.cu:548).  Dimers sit at
seeded uniform positions in a cube with >= ``spacing`` nm between all bead
centres (seeded rejection), random orientation angles U[-pi, pi), GDP
(curved) state.

Topology arrays follow read_PDB (src/preparator.cpp:249-355): harmonic
partners are beads of the same resid and chain with |i - j| < 2, encoded +j
when id_i > id_j else -j (unused slots -1); ``fixed`` = resid <= fix.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from ._abi import MtgParams

KB = 0.0019872041  # kcal/(mol K), src/mt.h:40
R_MON = 2.0
R_MT = 8.12
ZERO_CODE = 999999


# --------------------------------------------------------------- parameters
def derive_params(p: MtgParams) -> MtgParams:
    """gammaR, gammaTheta, varR, varTheta as src/preparator.cpp:209-219 computes them."""
    a = p.tea_a if p.hdi_on else R_MON
    p.gammaR = np.float32(6 * math.pi * p.viscosity * a)
    p.gammaTheta = np.float32(8 * math.pi * p.viscosity * R_MON ** 3)
    kb = np.float32(KB)
    p.varR = np.sqrt(np.float32(2.0) * kb * np.float32(p.Temp) * np.float32(p.dt) / np.float32(p.gammaR))
    p.varTheta = np.sqrt(np.float32(2.0) * kb * np.float32(p.Temp) * np.float32(p.dt) / np.float32(p.gammaTheta))
    return p


def default_params(seed: int = 1, **overrides) -> MtgParams:
    """Parameter set of the synthetic workloads.

    Force field from the reference's template/morse.conf (C = 300, B_psi =
    B_fi = 9125, B_theta = 90, theta0 GDP/GTP 0.2/0.0, LJ sigma 3.8 and scale
    0.1, seam coefficient 1) with Morse depths drawn from U[5, 15] kT and
    widths from U[2, 4] nm^-1 (seeded), LJ list cutoff 8 nm rebuilt every 10
    steps, 300 K, dt = 100 ps, barriers, walls and hydrolysis off, assembly
    mode on.  The viscosity defaults to the template's 2.85e4
    kcal ps/(mol nm^3): with water (128) the explicit Euler update is unstable
    at dt = 100 ps (C dt / gammaR ~ 6).
    """
    rng = np.random.default_rng(seed)
    kt = KB * 300.0
    p = MtgParams()
    p.dt = 100.0
    p.Temp = 300.0
    p.viscosity = 2.85e4
    p.alpha = 5.0
    p.freeze_temp = 1.0
    p.C = 300.0
    p.B_psi = 9125.0
    p.B_fi = 9125.0
    p.B_theta = 90.0
    p.psi_0 = 0.0
    p.fi_0 = 0.0
    p.theta0_gtp = 0.0
    p.theta0_gdp = 0.2
    p.D_long = float(rng.uniform(5, 15) * kt)
    p.A_long = float(rng.uniform(2, 4))
    p.D_lat = float(rng.uniform(5, 15) * kt)
    p.A_lat = float(rng.uniform(2, 4))
    p.seam_coeff = 1.0
    p.barrier = 0
    p.a_barr_long, p.r_barr_long, p.w_barr_long = 3.4, 0.4, 0.10 / (2 * math.sqrt(-2 * math.log(0.5)))
    p.a_barr_lat, p.r_barr_lat, p.w_barr_lat = 1.9, 0.4, 0.15 / (2 * math.sqrt(-2 * math.log(0.5)))
    p.lj_on = 1
    p.ljscale = 0.1
    p.ljsigma6 = float(np.float32(3.8) ** 6)
    p.ljpairscutoff = 8.0
    p.ljpairsupdatefreq = 10
    p.is_wall = 0
    p.rep_r = 80.0
    p.rep_eps = 0.005
    p.rep_leftborder = 0.0
    p.is_assembly = 1
    p.hdi_on = 0
    p.tea_a = 2.0
    p.tea_epsilon_freq = 10
    p.tea_capricious = 1
    p.tea_epsmax = 999.0
    p.rseed = 1234567
    for k, v in overrides.items():
        setattr(p, k, v)
    return derive_params(p)


# ------------------------------------------------------------ trajectories
@dataclasses.dataclass
class Trajectory:
    """One trajectory: per-bead arrays in template order."""

    coords: np.ndarray        # [n, 7] float32 x, y, z, fi, theta, psi, w
    mon_type: np.ndarray      # [n] int32
    resid: np.ndarray         # [n] int32
    chain: np.ndarray         # [n] int32 (chain code; -1 = extra 'X')
    atom_id: np.ndarray       # [n] int32
    extra: np.ndarray         # [n] uint8
    gtp: np.ndarray           # [n] int32
    zs: float = 160.0
    n_lattice: int = 0

    @property
    def n(self) -> int:
        return self.coords.shape[0]


def _rot_z_axis(fi, theta, psi):
    """Third column of R = Rz(psi) Ry(theta) Rx(fi) (the bead's z axis)."""
    sf, cf = np.sin(fi), np.cos(fi)
    st, ct = np.sin(theta), np.cos(theta)
    sp, cp = np.sin(psi), np.cos(psi)
    return np.stack([cp * st * cf + sp * sf, sp * st * cf - cp * sf, ct * cf], axis=-1)


def make_lattice(n_mon: int, radius: float = 12.0, psi_mode: str = "zero", tail: int = 0,
                 bend: float = 0.0, n_pf: int = 13):
    """Straight (optionally plus-end-bent) microtubule lattice, make_mt.py:29-66 semantics."""
    rows = []
    z_step = 6.0 / 13.0 * R_MON
    for k in range(n_pf):
        alpha = 2 * math.pi * k / 13.0
        for m in range(n_mon):
            from_end = n_mon - m
            if tail > 0 and from_end < tail:
                rad = radius + (tail - from_end) * 2 * R_MON * math.sin(bend)
                theta = bend
            else:
                rad = radius
                theta = 0.0
            x, y = rad * math.cos(-alpha), rad * math.sin(-alpha)
            z = 2 * R_MON * m + z_step * k
            psi = -alpha if psi_mode == "make_mt" else 0.0
            rows.append((x, y, z, 0.0, theta, psi, m % 2, m // 2 + 1, k, m + n_mon * k + 1))
    a = np.array(rows, dtype=np.float64).reshape(-1, 10)
    coords = np.zeros((a.shape[0], 7), np.float32)
    coords[:, :6] = a[:, :6]
    return coords, a[:, 6].astype(np.int32), a[:, 7].astype(np.int32), a[:, 8].astype(np.int32), \
        a[:, 9].astype(np.int32)


def place_free_dimers(rng, existing: np.ndarray, n_dimers: int, lo, hi, spacing: float = 4.0):
    """Seeded rejection placement of CA/CB dimers keeping >= spacing between all centres.

    Candidates are drawn in batches; a candidate is rejected when either bead
    is closer than ``spacing`` to an accepted bead, and conflicts inside a
    batch are resolved in draw order."""
    from scipy.spatial import cKDTree

    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    acc_pts = existing.astype(np.float64).reshape(-1, 3)
    placed_ca = np.zeros((0, 3))
    placed_ang = np.zeros((0, 3))
    rounds = 0
    while len(placed_ca) < n_dimers:
        rounds += 1
        if rounds > 200:
            raise RuntimeError("free tubulin placement failed: box too dense")
        need = n_dimers - len(placed_ca)
        k = max(64, int(need * 1.5))
        ca = rng.uniform(lo, hi, size=(k, 3))
        ang = rng.uniform(-math.pi, math.pi, size=(k, 3))
        cb = ca + 2 * R_MON * _rot_z_axis(ang[:, 0], ang[:, 1], ang[:, 2])
        ok = np.ones(k, bool)
        if len(acc_pts):
            tree = cKDTree(acc_pts)
            d1, _ = tree.query(ca)
            d2, _ = tree.query(cb)
            ok &= (d1 >= spacing) & (d2 >= spacing)
        idx = np.nonzero(ok)[0]
        pts = np.concatenate([ca[idx], cb[idx]])
        owner = np.concatenate([np.arange(len(idx)), np.arange(len(idx))])
        pairs = cKDTree(pts).query_pairs(spacing, output_type="ndarray") if len(pts) else np.zeros((0, 2), int)
        conflict = [[] for _ in range(len(idx))]
        for a, b in pairs:
            oa, ob = owner[a], owner[b]
            if oa != ob:
                conflict[max(oa, ob)].append(min(oa, ob))
        take = np.zeros(len(idx), bool)
        for c in range(len(idx)):
            if take.sum() >= need:
                break
            take[c] = not any(take[o] for o in conflict[c])
        sel = idx[take]
        placed_ca = np.concatenate([placed_ca, ca[sel]])
        placed_ang = np.concatenate([placed_ang, ang[sel]])
        acc_pts = np.concatenate([acc_pts, ca[sel], cb[sel]])
    return placed_ca[:n_dimers], placed_ang[:n_dimers]


def make_trajectory(n_mon: int, n_free: int, seed: int, radius: float = 12.0, psi_mode: str = "zero",
                    cube: float = 100.0, tail: int = 0, bend: float = 0.0, n_extra_dimers: int = 0,
                    spacing: float = 4.0, thermal: float = 0.0) -> Trajectory:
    """Lattice of 13 x n_mon monomers plus n_free free monomers (n_free/2 dimers).

    n_extra_dimers adds inert 'extra' dimers (chain X, src/preparator.cpp:289-301)
    parked away from the system.  ``thermal`` adds a seeded Gaussian jitter (nm,
    rad) to every coordinate, to move the lattice off its exact geometry."""
    rng = np.random.default_rng(seed)
    coords, mon, resid, chain, aid = make_lattice(n_mon, radius, psi_mode, tail, bend)
    n_dim = n_free // 2
    zc = 2 * R_MON * n_mon / 2
    lo = (-cube / 2, -cube / 2, zc - cube / 2)
    hi = (cube / 2, cube / 2, zc + cube / 2)
    ca, ang = place_free_dimers(rng, coords[:, :3], n_dim, lo, hi, spacing)
    cb = ca + 2 * R_MON * _rot_z_axis(ang[:, 0], ang[:, 1], ang[:, 2])
    fc = np.zeros((2 * n_dim, 7), np.float32)
    fc[0::2, :3] = ca
    fc[1::2, :3] = cb
    for c, col in ((0, 3), (1, 4), (2, 5)):
        fc[0::2, col] = ang[:, c]
        fc[1::2, col] = ang[:, c]
    fmon = np.tile(np.array([0, 1], np.int32), n_dim)
    fres = np.repeat(np.arange(n_dim, dtype=np.int32) + 10000, 2)
    fchain = np.repeat(np.arange(n_dim, dtype=np.int32) + 100, 2)
    fid = np.arange(2 * n_dim, dtype=np.int32) + len(aid) + 1
    parts = [(coords, mon, resid, chain, aid, np.zeros(len(mon), np.uint8), np.ones(len(mon), np.int32)),
             (fc, fmon, fres, fchain, fid, np.zeros(2 * n_dim, np.uint8), np.zeros(2 * n_dim, np.int32))]
    if n_extra_dimers:
        ec = np.zeros((2 * n_extra_dimers, 7), np.float32)
        ec[:, 0] = np.repeat(np.arange(n_extra_dimers) * 10.0 + 1000.0, 2)
        ec[1::2, 2] = 2 * 2 * R_MON / 2
        base = fid[-1] + 1 if len(fid) else len(aid) + 1
        parts.append((ec, np.tile(np.array([0, 1], np.int32), n_extra_dimers),
                      np.repeat(np.arange(n_extra_dimers, dtype=np.int32) + 20000, 2),
                      np.full(2 * n_extra_dimers, -1, np.int32),
                      np.arange(2 * n_extra_dimers, dtype=np.int32) + base,
                      np.ones(2 * n_extra_dimers, np.uint8), np.ones(2 * n_extra_dimers, np.int32)))
    cat = [np.concatenate([p[i] for p in parts]) for i in range(7)]
    t = Trajectory(coords=cat[0], mon_type=cat[1], resid=cat[2], chain=cat[3], atom_id=cat[4],
                   extra=cat[5], gtp=cat[6], zs=2 * R_MON * n_mon + 40.0, n_lattice=len(mon))
    if thermal > 0:
        jit = rng.normal(0.0, thermal, size=(t.n, 6)).astype(np.float32)
        jit[t.extra.astype(bool)] = 0
        t.coords[:, :6] += jit
    return t


def harmonic_topology(t: Trajectory, max_h: int = 1):
    """harmonicCount / harmonic as read_PDB builds them (src/preparator.cpp:325-355)."""
    n = t.n
    cnt = np.zeros(n, np.int32)
    harm = np.full(max_h * n, -1, np.int32)
    for i in range(n):
        for j in (i - 1, i + 1):
            if 0 <= j < n and t.resid[i] == t.resid[j] and t.chain[i] == t.chain[j]:
                if cnt[i] < max_h:
                    harm[max_h * i + cnt[i]] = j if t.atom_id[i] > t.atom_id[j] else -j
                cnt[i] += 1
    if cnt.max(initial=0) > max_h:
        raise ValueError("more harmonic partners than max_h")
    return cnt, harm


def fixed_mask(t: Trajectory, fix: int = 1):
    """fixed = resid <= fix (src/preparator.cpp:275-281)."""
    return (t.resid <= fix).astype(np.uint8)


# ----------------------------------------------------------------- batches
@dataclasses.dataclass
class Batch:
    """A batch of trajectories in CSR form (per-bead arrays over all beads)."""

    params: MtgParams
    offsets: np.ndarray       # [ntraj+1] int32
    coords: np.ndarray        # [nbeads, 7] float32
    mon_type: np.ndarray
    fixed: np.ndarray
    extra: np.ndarray
    gtp: np.ndarray
    on_tubule: np.ndarray
    harmonic_count: np.ndarray
    harmonic: np.ndarray      # [nbeads*max_h] local sign-encoded
    zs: np.ndarray            # [ntraj] float32
    max_h: int = 1
    max_long: int = 8
    max_lat: int = 16
    max_lj: int = 256
    uniform_ntot: int = 0     # > 0 when every trajectory shares one template

    @property
    def ntraj(self) -> int:
        return len(self.offsets) - 1

    @property
    def nbeads(self) -> int:
        return int(self.offsets[-1])

    def active_beads(self) -> int:
        return int(np.count_nonzero(self.extra == 0))


def batch_from_trajectories(params: MtgParams, trajs, fix: int = 1, max_h: int = 1, uniform: bool = False,
                            **caps) -> Batch:
    sizes = [t.n for t in trajs]
    offsets = np.zeros(len(trajs) + 1, np.int32)
    offsets[1:] = np.cumsum(sizes)
    hc, hh = zip(*[harmonic_topology(t, max_h) for t in trajs])
    b = Batch(
        params=params,
        offsets=offsets,
        coords=np.ascontiguousarray(np.concatenate([t.coords for t in trajs]).astype(np.float32)),
        mon_type=np.concatenate([t.mon_type for t in trajs]).astype(np.int32),
        fixed=np.concatenate([fixed_mask(t, fix) for t in trajs]).astype(np.uint8),
        extra=np.concatenate([t.extra for t in trajs]).astype(np.uint8),
        gtp=np.concatenate([t.gtp for t in trajs]).astype(np.int32),
        on_tubule=np.zeros(int(offsets[-1]), np.int32),
        harmonic_count=np.concatenate(hc).astype(np.int32),
        harmonic=np.concatenate(hh).astype(np.int32),
        zs=np.array([t.zs for t in trajs], np.float32),
        max_h=max_h,
        **caps,
    )
    if uniform:
        if len(set(sizes)) != 1:
            raise ValueError("uniform batch needs equal trajectory sizes")
        b.uniform_ntot = sizes[0]
    return b


def sub_batch(b: Batch, t0: int, t1: int) -> Batch:
    """Trajectories t0 .. t1-1 of a batch as a batch of their own (a copy of
    the parameters, offsets from 0, per-bead arrays sliced)."""
    import copy
    b0, b1 = int(b.offsets[t0]), int(b.offsets[t1])
    sub = Batch(params=copy.copy(b.params), offsets=(b.offsets[t0:t1 + 1] - b0).astype(np.int32),
                coords=b.coords[b0:b1].copy(), mon_type=b.mon_type[b0:b1].copy(), fixed=b.fixed[b0:b1].copy(),
                extra=b.extra[b0:b1].copy(), gtp=b.gtp[b0:b1].copy(), on_tubule=b.on_tubule[b0:b1].copy(),
                harmonic_count=b.harmonic_count[b0:b1].copy(),
                harmonic=b.harmonic[b.max_h * b0:b.max_h * b1].copy(), zs=b.zs[t0:t1].copy(), max_h=b.max_h,
                max_long=b.max_long, max_lat=b.max_lat, max_lj=b.max_lj, uniform_ntot=b.uniform_ntot)
    return sub


def uniform_batch(params: MtgParams, ntr: int, n_mon: int, n_free: int, seed: int = 0, **kw) -> Batch:
    """Ntr trajectories sharing one template topology, each with its own seeded
    free-tubulin placement (the template bead order is identical)."""
    trajs = [make_trajectory(n_mon, n_free, seed=seed * 100003 + t, **kw) for t in range(ntr)]
    return batch_from_trajectories(params, trajs, uniform=True)


def ragged_batch(params: MtgParams, ntraj: int, seed: int = 0, pf_range=(8, 120), free_range=(0, 2000),
                 cube: float = 150.0, bent_fraction: float = 0.3, bend_range=(0.1, 0.3), radius: float = 12.0,
                 **kw) -> Batch:
    """Uneven batch: PF length U{pf_range}, free count U{free_range} (rounded to
    dimers), a seeded fraction with a bent plus end."""
    rng = np.random.default_rng(seed)
    trajs = []
    for t in range(ntraj):
        n_mon = int(rng.integers(pf_range[0], pf_range[1] + 1))
        n_free = int(rng.integers(free_range[0], free_range[1] + 1)) // 2 * 2
        bent = rng.random() < bent_fraction
        bend = float(rng.uniform(*bend_range)) if bent else 0.0
        tail = min(n_mon, 6) if bent else 0
        trajs.append(make_trajectory(n_mon, n_free, seed=seed * 7919 + t, radius=radius, cube=cube,
                                     tail=tail, bend=bend, **kw))
    return batch_from_trajectories(params, trajs)
