"""CPU oracle of the updater's stride-step analytics (TEST INFRASTRUCTURE ONLY).

A numpy restatement of the reference's mt_length, hydrolyse and the counting
part of change_conc (src/updater.cpp), on the Coord AoS state
(x, y, z, fi, theta, psi, w) and per-bead flag arrays, for checking the
device kernels of mt_gb300/csrc/kernels_updater.cu.
"""
import numpy as np

R_MT = np.float32(8.12)          # src/mt.h:23
R_MON = np.float32(2.0)          # src/mt.h:24
ANG_THRES = np.float32(1.0)      # src/mt.h:29
R_THRES = R_MON * np.float32(8)  # src/mt.h:30


def on_tubule(coords):
    """The per-bead test of mt_length (src/updater.cpp:164-168), in FP32."""
    c = np.asarray(coords, np.float32)
    x, y, theta = c[:, 0], c[:, 1], c[:, 4]
    rad = np.sqrt(x * x + y * y)
    return (rad < R_MT + R_THRES) & (rad > np.float32(1.0)) & (np.cos(theta) > np.cos(ANG_THRES))


def decision_margin(coords):
    """Distance of each bead's mt_length decision from its thresholds (the
    test's margin filter: libm and CUDA cos may differ by an ulp)."""
    c = np.asarray(coords, np.float64)
    rad = np.sqrt(c[:, 0] ** 2 + c[:, 1] ** 2)
    return np.minimum.reduce([np.abs(rad - float(R_MT + R_THRES)), np.abs(rad - 1.0),
                              np.abs(np.cos(c[:, 4]) - np.cos(1.0))])


def mt_length(coords, offsets, on_cur, save_prev, on_prev):
    """mt_length (src/updater.cpp:154-227) after the compute loop's copy of
    on_tubule_cur to on_tubule_prev (src/compute_cuda.cu:1186) when
    save_prev: returns (mt_len per trajectory, on_cur, on_prev)."""
    on_prev = np.array(on_cur if save_prev else on_prev, np.int32)
    cur = on_tubule(coords).astype(np.int32)
    mt_len = np.array([cur[offsets[t]:offsets[t + 1]].sum() for t in range(len(offsets) - 1)], np.int32)
    return mt_len, cur, on_prev


def hydrolyse(offsets, gtp, extra, on_cur, on_prev, prob_source):
    """hydrolyse (src/updater.cpp:229-257) with rand()/RAND_MAX drawn from
    prob_source() in the reference's loop order (dimer outer, trajectory
    inner).  Returns (gtp, number of draws, events[(dimer, traj)] -> 1/2).
    Dimers are the bead pairs (2k, 2k+1) of a trajectory; an unpaired last
    bead is skipped (the reference's loop would touch the next trajectory's
    first bead there)."""
    gtp = np.array(gtp, np.int32)
    nt = len(offsets) - 1
    sizes = np.diff(offsets)
    max_dimers = int(sizes.max()) // 2 if nt else 0
    draws, events = 0, {}
    for k in range(max_dimers):
        for t in range(nt):
            if k >= sizes[t] // 2:   # dimer k = beads 2k, 2k+1 of the trajectory
                continue
            g = offsets[t] + 2 * k
            if gtp[g] == 1 and not extra[g] and on_cur[g] * on_prev[g] == 1:
                draws += 1
                if prob_source() < 0.02:
                    gtp[g] = gtp[g + 1] = 0
                    events[(k, t)] = 1
    for k in range(max_dimers):
        for t in range(nt):
            if k >= sizes[t] // 2:
                continue
            g = offsets[t] + 2 * k
            if gtp[g] == 0 and not extra[g] and on_cur[g] == 0 and on_prev[g] == 0:
                gtp[g] = gtp[g + 1] = 1
                events[(k, t)] = 2
    return gtp, draws, events


def count_extra(offsets, extra):
    """num_of_extra of change_conc (src/updater.cpp:103-108) per trajectory."""
    return np.array([int(np.count_nonzero(extra[offsets[t]:offsets[t + 1]])) for t in range(len(offsets) - 1)])


def hydrolyse_vec(offsets, gtp, extra, on_cur, on_prev, draw):
    """hydrolyse with numpy (the same decisions as `hydrolyse`): draw(n)
    returns the n candidates' numbers in the reference's order."""
    gtp = np.array(gtp, np.int32)
    offsets = np.asarray(offsets)
    nt = len(offsets) - 1
    half = np.diff(offsets) // 2
    md = int(half.max()) if nt else 0
    k, t = np.divmod(np.arange(md * nt), nt)          # slot order: dimer outer, trajectory inner
    ok = k < half[t]
    k, t = k[ok], t[ok]
    g = offsets[t] + 2 * k
    extra = np.asarray(extra).astype(bool)
    cand = (gtp[g] == 1) & ~extra[g] & (np.asarray(on_cur)[g] * np.asarray(on_prev)[g] == 1)
    n = int(cand.sum())
    hyd = np.zeros(len(g), bool)
    hyd[cand] = np.asarray(draw(n)) < 0.02
    gtp[g[hyd]] = 0
    gtp[g[hyd] + 1] = 0
    back = (gtp[g] == 0) & ~extra[g] & (np.asarray(on_cur)[g] == 0) & (np.asarray(on_prev)[g] == 0)
    gtp[g[back]] = 1
    gtp[g[back] + 1] = 1
    return gtp, n
