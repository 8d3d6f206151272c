"""Writes the golden fixtures of tests/golden/ from the reference's own kernels.

Runs the reference's kernel bodies compiled as host code
(oracle/_ref/libmtref.so, built by ``make -C oracle ref`` from the reference
tree) on small seeded systems and stores inputs and outputs as .npz files.
Regenerate with ``python tests/golden/make_golden.py`` where the reference
tree is present; the fixtures themselves travel with the repository.

Fixtures:
  rng.npz     ran2 seeds of rseed 1234567 and 256 rforce() draws of stream 0
  plain.npz   a 2-trajectory assembly-mode system: lists, forces, energies
              and one Euler-Maruyama step
  tea.npz     the same system with TEA on: epsilon/C_i pass, beta, one step
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mt_gb300 import synth  # noqa: E402
from mt_gb300._abi import ptr  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def system(tea: bool, **over):
    p = synth.default_params(seed=11, hdi_on=int(tea), tea_epsilon_freq=1 if tea else 10, **over)
    b = synth.uniform_batch(p, 2, 12, 40, seed=5, radius=8.12, psi_mode="make_mt", cube=40.0, thermal=0.05,
                            n_extra_dimers=2)
    return p, b


def params_dict(p):
    return {("param_" + k): np.array(v) for k, v in p.as_dict().items()}


def main():
    from oracle.reftree import reference_tree
    ref = reference_tree()
    if not ref:
        raise SystemExit("the reference tree is needed (MTG_REFERENCE_TREE or a checkout beside this repository)")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so", "ref", f"REF={ref}"],
                   check=True)
    # the reference's ran2 keeps static state: one seeding per process
    code = ("import sys, numpy as np; sys.path.insert(0, %r); from oracle import oracle as o;"
            "r = o.Oracle('ref'); s = r.generate_seeds(1234567, 64); st = s[:4].copy();"
            "g = r.rforce(st, 256); np.savez_compressed(%r, seeds=s, normals=g, state_after=st)")
    subprocess.run([sys.executable, "-c", code % (ROOT, os.path.join(HERE, "rng.npz"))], check=True)

    ref = orc.Oracle("ref")
    orc_f32 = orc.Oracle("orc")
    # ---------------------------------------------------------------- plain
    p, b = system(False)
    L = ref.lists(b, b.coords)
    f = ref.forces(b, b.coords, L)
    en = ref.energies(b, b.coords, L)
    seeds = orc_f32.generate_seeds(p.rseed, 2 * b.nbeads)
    r1 = b.coords.copy()
    f1 = f.copy()
    s1 = seeds.copy()
    v = orc._Views(b, 0, b.ntraj)
    ref._fn("integrate")(C.byref(p), C.byref(v.top), ptr(r1, C.c_float), ptr(f1, C.c_float), ptr(s1, C.c_uint32))
    np.savez_compressed(
        os.path.join(HERE, "plain.npz"), coords=b.coords, offsets=b.offsets, mon_type=b.mon_type, fixed=b.fixed,
        extra=b.extra, gtp=b.gtp, on_tubule=b.on_tubule, harmonic_count=b.harmonic_count, harmonic=b.harmonic,
        zs=b.zs, lj_count=L.lj_count, lj=L.lj, long_count=L.long_count, lon=L.lon, lat_count=L.lat_count,
        lat=L.lat, forces=f, energies=en, seeds=seeds, coords_after=r1, seeds_after=s1, **params_dict(p))
    # ------------------------------------------------------------------ TEA
    p, b = system(True)
    L = ref.lists(b, b.coords)
    f = ref.forces(b, b.coords, L)
    ci, eps = ref.tea_epsilon(b, b.coords)
    eps_t, beta, status = orc_f32.tea_beta(b, eps)
    seeds = orc_f32.generate_seeds(p.rseed, 2 * b.nbeads)
    rf = np.zeros((b.nbeads, 4), np.float32)
    mf = np.zeros_like(rf)
    cs = np.zeros_like(rf)
    f1 = f.copy()
    r1 = b.coords.copy()
    s1 = seeds.copy()
    v = orc._Views(b, 0, b.ntraj)
    ref._fn("tea_prepare")(C.byref(p), C.byref(v.top), ptr(f1, C.c_float), ptr(r1, C.c_float), ptr(s1, C.c_uint32),
                           ptr(rf, C.c_float), ptr(mf, C.c_float), ptr(cs, C.c_float))
    ref._fn("tea_integrate")(C.byref(p), C.byref(v.top), ptr(f1, C.c_float), ptr(r1, C.c_float),
                             ptr(s1, C.c_uint32), ptr(ci, C.c_float), ptr(beta, C.c_float), ptr(rf, C.c_float),
                             ptr(mf, C.c_float), ptr(cs, C.c_float))
    np.savez_compressed(
        os.path.join(HERE, "tea.npz"), coords=b.coords, offsets=b.offsets, mon_type=b.mon_type, fixed=b.fixed,
        extra=b.extra, gtp=b.gtp, on_tubule=b.on_tubule, harmonic_count=b.harmonic_count, harmonic=b.harmonic,
        zs=b.zs, lj_count=L.lj_count, lj=L.lj, long_count=L.long_count, lon=L.lon, lat_count=L.lat_count,
        lat=L.lat, forces=f, tea_ci=ci, tea_eps=eps, eps_traj=eps_t, beta=beta, beta_status=np.array(status),
        seeds=seeds, rforce=rf, coords_after=r1, seeds_after=s1, **params_dict(p))
    for name in ("rng.npz", "plain.npz", "tea.npz"):
        print(name, os.path.getsize(os.path.join(HERE, name)), "bytes")


if __name__ == "__main__":
    main()
