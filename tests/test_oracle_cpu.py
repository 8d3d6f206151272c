"""The CPU oracle against the golden fixtures written from the reference's own
kernels (tests/golden/make_golden.py), and, where the reference tree is
present, against those kernels directly on further seeded cases."""
import numpy as np
import pytest

from helpers import with_lone_monomers, golden_batch, rel_norm, small_system, system_with_margin

GOLD = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden")


def load(name):
    return np.load(f"{GOLD}/{name}")


def test_rng_matches_golden(oracle_lib):
    d = load("rng.npz")
    o = oracle_lib.Oracle("orc")
    seeds = o.generate_seeds(1234567, 64)
    assert np.array_equal(seeds, d["seeds"])            # ran2 seeding: bit-exact
    st = seeds[:4].copy()
    g = o.rforce(st, 256)
    assert np.array_equal(st, d["state_after"])         # HybridTaus integer stream: bit-exact
    np.testing.assert_allclose(g, d["normals"], rtol=0, atol=2e-6)
    assert np.all(seeds >= 128)                         # the reference redraws components < 128


def _lists_equal(L, d):
    for cnt, arr, cap, kc, ka in ((L.lj_count, L.lj, L.max_lj, "lj_count", "lj"),
                                  (L.long_count, L.lon, L.max_long, "long_count", "lon"),
                                  (L.lat_count, L.lat, L.max_lat, "lat_count", "lat")):
        assert np.array_equal(cnt, d[kc]), kc
        for i in range(len(cnt)):
            assert np.array_equal(arr[cap * i:cap * i + cnt[i]], d[ka][cap * i:cap * i + cnt[i]]), (ka, i)


def test_plain_matches_golden(oracle_lib):
    d = load("plain.npz")
    b = golden_batch(d)
    o = oracle_lib.Oracle("orc")
    L = o.lists(b, b.coords)
    _lists_equal(L, d)
    f = o.forces(b, b.coords, L)
    for c in range(6):
        assert rel_norm(f[:, c], d["forces"][:, c]) < 1e-5, c
    en = o.energies(b, b.coords, L)
    np.testing.assert_allclose(en.sum(0), d["energies"].sum(0), rtol=1e-5, atol=1e-4)
    # one Euler-Maruyama step from the same seeds
    x, _, s, _, status, _, _ = o.run(b, b.coords, d["seeds"], 1, 1, L=L)
    assert status == 0
    assert np.array_equal(s, d["seeds_after"])
    np.testing.assert_allclose(x[:, :6], d["coords_after"][:, :6], rtol=0, atol=2e-4)


def test_tea_matches_golden(oracle_lib):
    d = load("tea.npz")
    b = golden_batch(d)
    o = oracle_lib.Oracle("orc")
    ci, eps = o.tea_epsilon(b, b.coords)
    assert rel_norm(ci, d["tea_ci"]) < 1e-5
    assert rel_norm(eps, d["tea_eps"]) < 1e-5
    eps_t, beta, status = o.tea_beta(b, eps)
    np.testing.assert_allclose(eps_t, d["eps_traj"], rtol=1e-5)
    np.testing.assert_allclose(beta, d["beta"], rtol=1e-5)
    L = o.lists(b, b.coords)
    x, _, s, _, status, _, _ = o.run(b, b.coords, d["seeds"], 0, 1, L=L)
    assert status == 0
    assert np.array_equal(s, d["seeds_after"])          # TEA consumes both streams of every bead
    np.testing.assert_allclose(x[:, :6], d["coords_after"][:, :6], rtol=0, atol=5e-4)


def test_fp64_oracle_close_to_fp32(oracle_lib):
    b = small_system(seed=3)
    o32, o64 = oracle_lib.Oracle("orc", "f32"), oracle_lib.Oracle("orc", "f64")
    L = o32.lists(b, b.coords)
    f32, f64 = o32.forces(b, b.coords, L), o64.forces(b, b.coords, L)
    for c in range(6):
        assert rel_norm(f32[:, c], f64[:, c]) < 1e-5


ref_only = pytest.mark.skipif(not __import__("oracle.oracle", fromlist=["x"]).ref_available(),
                              reason="reference harness not built (needs the reference tree)")


@ref_only
@pytest.mark.parametrize("case", ["default", "walls_barrier_seam", "gdp_ontubule", "odd_pf", "lone_monomers",
                                  "lj_off", "lj_cut_5nm"])
def test_oracle_matches_reference_kernels(oracle_lib, case):
    over = {}
    if case == "walls_barrier_seam":
        over = dict(is_wall=1, rep_r=9.0, barrier=1, seam_coeff=1.7)
    if case == "lj_off":
        over = dict(lj_on=0)
    if case == "lj_cut_5nm":
        over = dict(ljpairscutoff=5.0)
    b = system_with_margin(seed=7, **over) if case != "odd_pf" else small_system(seed=9, n_mon=11)
    if case == "lone_monomers":
        b = with_lone_monomers(b)
    if case == "gdp_ontubule":
        rng = np.random.default_rng(4)
        b.gtp[:] = rng.integers(0, 2, b.nbeads)
        b.on_tubule[:] = rng.integers(0, 2, b.nbeads)
        b.params.barrier = 1
    o, r = oracle_lib.Oracle("orc"), oracle_lib.Oracle("ref")
    Lo, Lr = o.lists(b, b.coords), r.lists(b, b.coords)
    for k in ("lj", "long", "lat"):
        assert Lo.as_lists(k) == Lr.as_lists(k), k
    fo, fr = o.forces(b, b.coords, Lo), r.forces(b, b.coords, Lr)
    for c in range(6):
        assert rel_norm(fo[:, c], fr[:, c]) < 1e-5, c
    eo, er = o.energies(b, b.coords, Lo), r.energies(b, b.coords, Lr)
    np.testing.assert_allclose(eo.sum(0), er.sum(0), rtol=2e-5, atol=1e-3)


@ref_only
def test_zero_code_lateral_partner(oracle_lib):
    """Bead 0 as a lateral partner is encoded +-999999 (src/compute_cuda.cu:646-658)."""
    b = system_with_margin(seed=7)
    L = oracle_lib.Oracle("ref").lists(b, b.coords)
    codes = {v for lst in L.as_lists("lat") for v in lst}
    assert 999999 in codes or -999999 in codes
    Lo = oracle_lib.Oracle("orc").lists(b, b.coords)
    assert Lo.as_lists("lat") == L.as_lists("lat")
