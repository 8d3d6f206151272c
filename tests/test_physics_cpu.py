"""Physics checks of the algorithm on the CPU oracle (FP64 build; no GPU):
translational forces are minus the gradient of the energy (harmonic, Morse,
LJ and barrier terms; src/compute_cuda.cu:32-525 against :676-911), the RPY
mobility tensor of the TEA path is symmetric and positive definite, also
with overlapping beads (src/bdhitea_kernel.cu:38-58), and the noise of the
Euler-Maruyama update gives free diffusion at the set temperature."""
import numpy as np

from helpers import system_with_margin
from mt_gb300 import synth
from test_tea_farfield_cpu import rpy_blocks


def test_forces_are_minus_the_energy_gradient(oracle_lib):
    b = system_with_margin(seed=31, barrier=1)
    o = oracle_lib.Oracle("orc", "f64")
    x0 = b.coords.astype(np.float64)
    L = o.lists(b, x0)
    f = o.forces(b, x0, L)
    rng = np.random.default_rng(0)
    beads = rng.choice(np.nonzero(b.extra == 0)[0], 24, replace=False)
    h = 1e-4
    fd, an = [], []
    for i in beads:
        for a in range(3):
            xp, xm = x0.copy(), x0.copy()
            xp[i, a] += h
            xm[i, a] -= h
            up = o.energies(b, xp, L).sum()
            um = o.energies(b, xm, L).sum()
            fd.append(-(up - um) / (2 * h))
            an.append(f[i, a])
    fd, an = np.array(fd), np.array(an)
    assert np.linalg.norm(fd - an) / np.linalg.norm(an) < 1e-6, (fd[:6], an[:6])


def test_rpy_tensor_symmetric_positive_definite():
    rng = np.random.default_rng(1)
    for spread in (3.0, 10.0):            # 3 nm: many overlapping pairs (r < 2a = 4 nm)
        x = rng.uniform(-spread, spread, size=(40, 3))
        cii, crr, u, r = rpy_blocks(x)
        n = len(x)
        D = cii[..., None, None] * np.eye(3) + crr[..., None, None] * u[..., :, None] * u[..., None, :]
        D[np.arange(n), np.arange(n)] = np.eye(3)                 # D_ii / D_ii
        M = D.transpose(0, 2, 1, 3).reshape(3 * n, 3 * n)
        assert np.allclose(M, M.T, atol=1e-12)
        assert (r[np.triu_indices(n, 1)] < 4.0).any() or spread > 5
        assert np.linalg.eigvalsh(M).min() > 0.0


def test_free_diffusion_temperature(oracle_lib):
    """All interactions off: every step moves a bead by varR * N(0,1) per axis,
    so gammaR <dx^2> / (2 kB dt) is the set temperature."""
    p = synth.default_params(seed=3, C=0.0, D_long=0.0, D_lat=0.0, B_psi=0.0, B_fi=0.0, B_theta=0.0, lj_on=0,
                             is_assembly=0)
    b = synth.uniform_batch(p, 4, 4, 400, seed=3, cube=200.0)
    o = oracle_lib.Oracle("orc", "f64")
    seeds = o.generate_seeds(p.rseed, 2 * b.nbeads)
    x = b.coords.astype(np.float64)
    moving = (b.extra == 0) & (b.fixed == 0)
    d2 = []
    for k in range(20):
        xn, _, seeds, _, st, _, _ = o.run(b, x, seeds, k, 1)
        assert st == 0
        d2.append((xn[moving, :3] - x[moving, :3]) ** 2)
        x = xn
    msd = np.concatenate(d2).mean()
    temp = p.gammaR * msd / (2 * synth.KB * p.dt)
    assert abs(temp / p.Temp - 1) < 0.02, temp


def test_angular_forces_are_minus_the_energy_gradient(oracle_lib):
    """With all bending equilibria at zero the generalised forces of the
    three Euler angles (bending + site torques projected on the Euler axes)
    are minus the angle derivatives of the energy.  With a non-zero theta0
    they are not: the reference's bending energy and force use differently
    ordered angle differences (src/compute_cuda.cu:158-164 against :751-756)."""
    b = system_with_margin(seed=31, theta0_gtp=0.0, theta0_gdp=0.0, psi_0=0.0, fi_0=0.0)
    o = oracle_lib.Oracle("orc", "f64")
    x0 = b.coords.astype(np.float64)
    L = o.lists(b, x0)
    f = o.forces(b, x0, L)
    beads = np.random.default_rng(0).choice(np.nonzero(b.extra == 0)[0], 12, replace=False)
    h = 1e-5
    for col in (3, 4, 5):                   # fi, theta, psi
        fd = []
        for i in beads:
            xp, xm = x0.copy(), x0.copy()
            xp[i, col] += h
            xm[i, col] -= h
            fd.append(-(o.energies(b, xp, L).sum() - o.energies(b, xm, L).sum()) / (2 * h))
        an = f[beads, col]
        assert np.linalg.norm(np.array(fd) - an) / np.linalg.norm(an) < 1e-7, col
