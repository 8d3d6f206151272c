"""Stride-step hooks of the reference's updater on the device-resident state.

Mirrors mt_length, hydrolyse and change_conc (src/updater.cpp:97-257) on top
of the engine's analytics kernels (mtg_mt_length, mtg_hydrolysis_candidates /
mtg_hydrolyse, mtg_count_extra / mtg_set_beads): the coordinates stay on the
GPU; only per-trajectory counts, the random numbers and the few re-inserted
dimers cross the bus.  Random numbers come from a caller-supplied source of
rand()-like integers in [0, rand_max], so a caller that passes the C
library's rand() reproduces the reference's choices.
"""
from __future__ import annotations

import numpy as np

R_MON = 2.0
PF_NUMBER = 13


class Updater:
    def __init__(self, engine, rand, rand_max: int = 2147483647, out=print):
        self.e = engine
        self.rand = rand
        self.rand_max = rand_max
        self.out = out
        self.mt_len = np.zeros(engine.nt, np.int32)

    def mt_length(self, step: int, save_prev: bool, mt_len_file: str | None = None):
        """on_tubule flags and per-trajectory counts (src/updater.cpp:154-227)."""
        self.mt_len = self.e.mt_length(save_prev)
        for t, n in enumerate(self.mt_len):
            self.out(f"tubule[{t}]: {n}")
        if mt_len_file:
            with open(mt_len_file, "w" if step == 0 else "a") as f:
                f.write(f"{step}\t" + "".join(f"{2 * R_MON * float(n) / PF_NUMBER:f}\t" for n in self.mt_len) + "\n")
        return self.mt_len

    def hydrolyse(self):
        """GTP hydrolysis and return to GTP (src/updater.cpp:229-257)."""
        n = self.e.hydrolysis_candidates()
        prob = np.array([self.rand() / float(self.rand_max) for _ in range(n)], np.float64)
        nh, nr, ev = self.e.hydrolyse(prob, events=True)
        for kind, text in ((1, "Hydrolysis occured"), (2, "Transition to GTP occured")):
            for k, t in zip(*np.nonzero(ev == kind)):
                self.out(f"*** {text} to dimer # {k} trajectory #{t} ***")
        return nh, nr

    def change_conc(self, conc: float, rep_r: float, zs, rep_leftborder: float, mon_type, ntot: int):
        """Constant free-tubulin concentration (src/updater.cpp:97-152) for a
        uniform batch of `ntot` beads per trajectory: re-inserts extra dimers
        at random (x, y) in the cylinder of radius rep_r.  Returns the number
        of re-inserted dimers."""
        n_extra = self.e.count_extra()
        _, extra, _, _ = self.e.download_flags()
        state = None
        flag = 0
        for tr in range(self.e.nt):
            num_extra = int(n_extra[tr])
            vol = float(np.float32(3.14 * rep_r * rep_r * zs[tr]))
            n_free = (ntot - int(self.mt_len[tr]) - num_extra) // 2
            while 1.0e7 * n_free / 6.0 < conc * vol:
                for i in range(0, ntot, 2):
                    g = i + tr * ntot
                    if extra[g] and mon_type[i] == 0:
                        extra[g] = extra[g + 1] = 0
                        while True:
                            x = rep_r - 2 * (self.rand() % int(rep_r))
                            y = rep_r - 2 * (self.rand() % int(rep_r))
                            if x * x + y * y <= rep_r * rep_r:
                                num_extra -= 2
                                break
                        z = zs[tr] + rep_leftborder + 3 * 2 * R_MON
                        if state is None:
                            state = self.e.download_state()
                        c = state[[g, g + 1]].copy()
                        c[:, 0:3] = [[x, y, z], [x, y, z + 2 * R_MON]]
                        self.e.set_beads([g, g + 1], c, extra=np.zeros(2, np.uint8))
                        flag += 1
                        break
                n_free += 1
                if num_extra == 0:
                    self.out(f"No more extra particles for trajectory[{tr}]!")
                    break
            self.out(f"Concentration for tajectory[{tr}]: {1.0e7 * n_free / (6.0 * vol):f} [muMole / L]")
        return flag
