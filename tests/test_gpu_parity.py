"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on
identical inputs and seeds.

Bars: integer/index work bit-exact (HybridTaus streams, ran2 seeds, pair
lists on states whose list decisions sit > 2e-4 nm from every cutoff);
forces and energies within 1e-5 relative (norm over the array, per
component) in FP32; multi-step states within the FP32 drift stated per test.
"""
import numpy as np
import pytest

from helpers import rel_norm, small_system, system_with_margin, with_lone_monomers

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5


def make_engine(engine_mod, b, **kw):
    e = engine_mod.Engine(b, **kw)
    e.upload_state(b.coords)
    return e


def test_seeds_match_reference_ran2(engine_mod, oracle_lib):
    b = small_system(seed=2)
    e = make_engine(engine_mod, b)
    o = oracle_lib.Oracle("orc")
    assert np.array_equal(e.download_rng(), o.generate_seeds(b.params.rseed, 2 * b.nbeads))
    e.close()


@pytest.mark.parametrize("ragged", [False, True])
@pytest.mark.parametrize("method", [1, 2])
def test_lists_bit_exact(engine_mod, oracle_lib, ragged, method):
    b = system_with_margin(seed=5, ntr=3)
    e = make_engine(engine_mod, b, force_ragged=ragged)
    e.set_list_method(method)
    e.rebuild_pairs()
    L = oracle_lib.Oracle("orc").lists(b, b.coords)
    for k in ("lj", "long", "lat"):
        assert e.list_of_lists(k) == L.as_lists(k), k
    e.close()


def test_lists_golden(engine_mod):
    """Lists of the fixture written from the reference's own pairs/LJ kernels."""
    from helpers import golden_batch
    d = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "plain.npz"))
    b = golden_batch(d)
    e = make_engine(engine_mod, b)
    e.rebuild_pairs()
    got = e.lists()
    for kind, kc, ka in (("lj", "lj_count", "lj"), ("long", "long_count", "lon"), ("lat", "lat_count", "lat")):
        cnt, arr, cap = got[kind]
        assert np.array_equal(cnt, d[kc]), kind
        for i in range(b.nbeads):
            assert np.array_equal(arr[cap * i:cap * i + cnt[i]], d[ka][cap * i:cap * i + cnt[i]]), (kind, i)
    e.close()


@pytest.mark.parametrize("case", ["default", "walls_barrier_seam", "gdp_ontubule", "static_lists", "lone_monomers"])
def test_forces_and_energies(engine_mod, oracle_lib, case):
    over = {}
    if case == "walls_barrier_seam":
        over = dict(is_wall=1, rep_r=9.0, barrier=1, seam_coeff=1.7)
    b = system_with_margin(seed=8, **over)
    if case == "lone_monomers":
        b = with_lone_monomers(b)
    if case == "gdp_ontubule":
        rng = np.random.default_rng(4)
        b.gtp[:] = rng.integers(0, 2, b.nbeads)
        b.on_tubule[:] = rng.integers(0, 2, b.nbeads)
        b.params.barrier = 1
    o32, o64 = oracle_lib.Oracle("orc", "f32"), oracle_lib.Oracle("orc", "f64")
    L = o32.lists(b, b.coords)
    if case == "static_lists":
        b.params.is_assembly = 0
        e = make_engine(engine_mod, b, static_lists=L)
        e.rebuild_pairs()   # LJ only; the static lists stay
    else:
        e = make_engine(engine_mod, b)
        e.rebuild_pairs()
        for k in ("lj", "long", "lat"):
            assert e.list_of_lists(k) == L.as_lists(k), k
    f = e.compute_forces()
    fo, f64 = o32.forces(b, b.coords, L), o64.forces(b, b.coords, L)
    for c in range(6):
        err = rel_norm(f[:, c], fo[:, c])
        assert err < FORCE_RTOL, (c, err, rel_norm(f[:, c], f64[:, c]))
    tot, per = e.energies(per_bead=True)
    eo = o32.energies(b, b.coords, L)
    for t in range(b.ntraj):
        sl = slice(int(b.offsets[t]), int(b.offsets[t + 1]))
        np.testing.assert_allclose(tot[t], eo[sl].sum(0), rtol=1e-5, atol=1e-3)
    assert rel_norm(per, eo) < 1e-5
    e.close()


def test_one_step_matches_oracle(engine_mod, oracle_lib):
    b = system_with_margin(seed=11)
    o = oracle_lib.Oracle("orc")
    seeds = o.generate_seeds(b.params.rseed, 2 * b.nbeads)
    e = make_engine(engine_mod, b)
    e.step(0, 1)
    x = e.download_state()
    xo, _, so, _, st, _, _ = o.run(b, b.coords, seeds, 0, 1)
    assert st == 0
    assert np.array_equal(e.download_rng(), so)          # streams consumed by moving beads only
    np.testing.assert_allclose(x[:, :6], xo[:, :6], rtol=0, atol=5e-5)


def test_zero_temperature_trajectory(engine_mod, oracle_lib):
    """Temp = 0 makes the update deterministic (varR = varTheta = 0); 30 steps
    with three list rebuilds stay within FP32 drift of the oracle."""
    b = system_with_margin(seed=12, Temp=0.0)
    o = oracle_lib.Oracle("orc")
    seeds = o.generate_seeds(b.params.rseed, 2 * b.nbeads)
    e = make_engine(engine_mod, b)
    e.step(0, 30)
    x = e.download_state()
    xo = o.run(b, b.coords, seeds, 0, 30)[0]
    np.testing.assert_allclose(x[:, :3], xo[:, :3], rtol=0, atol=2e-3)
    np.testing.assert_allclose(x[:, 3:6], xo[:, 3:6], rtol=0, atol=2e-3)


def test_graph_replay_equals_single_steps(engine_mod):
    b = small_system(seed=13)
    e1 = make_engine(engine_mod, b)
    e1.step(0, 25)                       # two graph replays + tail
    e2 = make_engine(engine_mod, b)
    for s in range(25):
        e2.step(s, 1)
    assert np.array_equal(e1.download_state(), e2.download_state())
    assert np.array_equal(e1.download_rng(), e2.download_rng())


def test_ragged_batch_forces(engine_mod, oracle_lib):
    from mt_gb300 import synth
    p = synth.default_params(seed=3)
    b = synth.ragged_batch(p, 5, seed=3, pf_range=(4, 14), free_range=(0, 60), cube=50.0, radius=8.12,
                           psi_mode="make_mt", thermal=0.05)
    e = make_engine(engine_mod, b)
    e.rebuild_pairs()
    o = oracle_lib.Oracle("orc")
    L = o.lists(b, b.coords)
    f = e.compute_forces()
    fo = o.forces(b, b.coords, L)
    for c in range(6):
        assert rel_norm(f[:, c], fo[:, c]) < FORCE_RTOL
    tot = e.energies()
    eo = o.energies(b, b.coords, L)
    for t in range(b.ntraj):
        sl = slice(int(b.offsets[t]), int(b.offsets[t + 1]))
        np.testing.assert_allclose(tot[t], eo[sl].sum(0), rtol=1e-5, atol=1e-3)


def test_tea_update_and_step(engine_mod, oracle_lib):
    b = system_with_margin(seed=14, tea=True, tea_epsilon_freq=1)
    o32, o64 = oracle_lib.Oracle("orc", "f32"), oracle_lib.Oracle("orc", "f64")
    e = make_engine(engine_mod, b)
    eps, beta, ci, rc = e.tea_update()
    assert rc == 0
    ci_o, eps_o = o32.tea_epsilon(b, b.coords)
    eps_t, beta_o, st = o32.tea_beta(b, eps_o)
    assert rel_norm(ci[:, :3], ci_o[:, :3]) < 1e-5
    np.testing.assert_allclose(eps, eps_t, rtol=1e-5)
    np.testing.assert_allclose(beta, beta_o, rtol=1e-5)
    # one TEA step from identical state and seeds
    seeds = o32.generate_seeds(b.params.rseed, 2 * b.nbeads)
    e2 = make_engine(engine_mod, b)
    e2.step(0, 1)
    x = e2.download_state()
    xo, _, so, _, st, _, _ = o32.run(b, b.coords, seeds, 0, 1)
    assert st == 0
    assert np.array_equal(e2.download_rng(), so)         # TEA draws both streams of every bead
    np.testing.assert_allclose(x[:, :6], xo[:, :6], rtol=0, atol=1e-4)


def test_overflow_reported(engine_mod):
    b = small_system(seed=15)
    b.max_lj = 4
    e = make_engine(engine_mod, b)
    with pytest.raises(engine_mod.MtgError) as ex:
        e.rebuild_pairs()
    assert ex.value.code == -3


def test_nonfinite_energy_reported(engine_mod):
    b = small_system(seed=16)
    c = b.coords.copy()
    c[5, 0] = np.nan
    e = engine_mod.Engine(b)
    e.upload_state(c)
    e.rebuild_pairs()
    with pytest.raises(engine_mod.MtgError) as ex:
        e.energies()
    assert ex.value.code == -4
    # the context stays usable
    e.upload_state(b.coords)
    e.rebuild_pairs()
    assert np.all(np.isfinite(e.energies()))


def test_tea_epsmax_reported(engine_mod):
    b = small_system(seed=17, tea=True, tea_epsilon_freq=1, tea_epsmax=1e-6)
    e = make_engine(engine_mod, b)
    assert e.step_raw(0, 1) == -5


def test_kernel_timing_in_graphs(engine_mod):
    """Per-kernel events recorded inside the replayed graphs are readable."""
    b = small_system(seed=18)
    e = make_engine(engine_mod, b)
    e.set_kernel_timing(True)
    e.step(0, 10)                 # capture + one replay
    e.kernel_times(reset=True)
    ms = e.step_timed(10, 10)
    kt = e.kernel_times()
    assert kt["rebuild"][1] == 1 and kt["step_plain"][1] == 10
    assert 0 < kt["step_plain"][0] <= ms
    e.set_kernel_timing(False)
    assert e.step_timed(20, 15) > 0   # graph + direct launches without timing


def test_cell_lists_equal_tile_lists_on_a_large_batch(engine_mod):
    """The cell-list and the tiled rebuild evaluate identical FP32 expressions,
    so their lists agree exactly on any state (no cutoff margin needed)."""
    from mt_gb300 import synth
    p = synth.default_params(seed=4)
    b = synth.uniform_batch(p, 8, 40, 1000, seed=4, cube=100.0)
    e = make_engine(engine_mod, b)
    e.step(0, 20)                      # move off the generated geometry
    e.set_list_method(1)
    e.rebuild_pairs()
    tiles = e.lists()
    e.set_list_method(2)
    e.rebuild_pairs()
    cells = e.lists()
    for k in ("lj", "long", "lat"):
        assert np.array_equal(tiles[k][0], cells[k][0]), k
        cnt, arr, cap = cells[k]
        for i in range(e.nb):
            assert np.array_equal(arr[cap * i:cap * i + cnt[i]], tiles[k][1][cap * i:cap * i + cnt[i]]), (k, i)


def test_autotune_leaves_the_simulation_unchanged(engine_mod):
    """The autotuner restores the state and noise streams after its trials,
    and the plain-path kernels give identical results for every launch shape."""
    b = small_system(seed=19, ntr=3)
    e1 = make_engine(engine_mod, b)
    res = e1.autotune(0, 10)
    assert res["tuning"]["step_block"] in (64, 128, 256)
    e1.step(0, 20)
    e2 = make_engine(engine_mod, b)
    e2.step(0, 20)
    assert np.array_equal(e1.download_state(), e2.download_state())
    assert np.array_equal(e1.download_rng(), e2.download_rng())


def _restart_roundtrip(engine_mod, b, tmp_path, n1, n2, mutate=None):
    """n1 + n2 steps straight vs n1 steps, restart file, a fresh engine, n2 steps."""
    e1 = engine_mod.Engine(b)
    e1.upload_state(b.coords)
    if mutate:
        mutate(e1)
    e1.step(0, n1 + n2)
    ref_state, ref_rng = e1.download_state(), e1.download_rng()
    e1.close()
    e2 = engine_mod.Engine(b)
    e2.upload_state(b.coords)
    if mutate:
        mutate(e2)
    e2.step(0, n1)
    path = str(tmp_path / "run.mtgrst")
    e2.write_restart(path, n1)
    e2.close()
    e3 = engine_mod.Engine(b)
    first = e3.read_restart(path)
    assert first == n1
    e3.step(first, n2)
    assert np.array_equal(e3.download_state(), ref_state)
    assert np.array_equal(e3.download_rng(), ref_rng)
    e3.close()


def test_restart_is_bit_exact_plain(engine_mod, tmp_path):
    b = small_system(seed=41)
    # resume in the middle of a pair-list period (the lists come from the file)
    _restart_roundtrip(engine_mod, b, tmp_path, 15, 17,
                       mutate=lambda e: e.set_gtp(np.where(np.arange(b.nbeads) % 3 == 0, 1, 0)))


def test_restart_is_bit_exact_tea(engine_mod, tmp_path):
    b = small_system(seed=42, tea=True, tea_epsilon_freq=5)
    _restart_roundtrip(engine_mod, b, tmp_path, 13, 12)   # between two epsilon steps


def test_restart_rejects_other_systems_and_corruption(engine_mod, tmp_path):
    b = small_system(seed=43)
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.step(0, 3)
    path = tmp_path / "a.mtgrst"
    e.write_restart(str(path), 3)
    e.close()
    other = engine_mod.Engine(small_system(seed=43, n_free=60))
    with pytest.raises(engine_mod.MtgError):
        other.read_restart(str(path))
    other.close()
    raw = bytearray(path.read_bytes())
    raw[100] ^= 0x40
    bad = tmp_path / "bad.mtgrst"
    bad.write_bytes(bytes(raw))
    e = engine_mod.Engine(b)
    with pytest.raises(engine_mod.MtgError):
        e.read_restart(str(bad))
    e.close()


def test_tea_split_j_range_matches(engine_mod):
    """Splitting each trajectory's j range over several CTAs (tea_jparts)
    changes only the summation order of the all-pairs kernels."""
    b = system_with_margin(seed=44, tea=True, tea_epsilon_freq=2, n_free=300)
    ref = None
    for jp in (1, 2, 3, 4):
        e = make_engine(engine_mod, b)
        t = e.tuning()
        e.set_tuning(t["list_method"], t["step_block"], 2, jp)
        e.step(0, 4)
        x = e.download_state()
        rng = e.download_rng()
        if ref is None:
            ref = (x, rng)
        else:
            assert np.array_equal(rng, ref[1])
            np.testing.assert_allclose(x[:, :6], ref[0][:, :6], rtol=0, atol=2e-5)
        e.close()


def test_tea_split_tail_on_a_large_batch(engine_mod):
    """With more than two waves of work items the TEA launchers run the first
    items whole and split only the last ones over several CTAs; the result
    equals the unsplit launch up to the summation order."""
    from mt_gb300 import synth
    p = synth.default_params(seed=45, hdi_on=1, tea_a=2.0, tea_epsilon_freq=2)
    b = synth.uniform_batch(p, 48, 100, 3000, seed=45, cube=150.0)
    assert b.nbeads // 48 // 128 * 48 >= 2 * 5 * 152   # items >= two waves of 5 CTAs on 152 SMs
    ref = None
    for jp in (1, 3):
        e = make_engine(engine_mod, b)
        t = e.tuning()
        e.set_tuning(t["list_method"], t["step_block"], 4, jp)
        e.step(0, 2)
        x = e.download_state()
        rng = e.download_rng()
        if ref is None:
            ref = (x, rng)
        else:
            assert np.array_equal(rng, ref[1])
            # lattice z reaches 400 nm, where one FP32 ulp is 3.05e-5
            np.testing.assert_allclose(x[:, :6], ref[0][:, :6], rtol=2.5e-7, atol=2e-5)
        e.close()


def test_graph_kernel_launch_count(engine_mod):
    """Every replay of a list-period graph adds that graph's kernel nodes:
    at least one fused step per MD step plus the list rebuild."""
    b = small_system(seed=46)
    e = make_engine(engine_mod, b)
    period = int(b.params.ljpairsupdatefreq)
    e.step(0, period)                      # captures the graph and replays it once
    n1 = e.graph_kernel_launches(reset=True)
    e.step(period, 2 * period)             # two more replays
    n2 = e.graph_kernel_launches(reset=True)
    assert n1 >= period + 1, n1
    assert n2 == 2 * n1, (n1, n2)
    assert e.graph_kernel_launches() == 0
    e.step(3 * period, 3)                  # shorter than a period: no graph
    assert e.graph_kernel_launches() == 0
    e.close()


def test_tea_ragged_batch_matches_oracle(engine_mod, oracle_lib):
    """TEA on an uneven batch (trajectories of 52 to ~480 beads, several
    128-bead chunks each): epsilon, beta, C_i and one step against the
    oracle, with whole and with split j ranges."""
    from helpers import cutoff_margin
    from mt_gb300 import synth
    for seed in range(70, 120):
        p = synth.default_params(seed=seed, hdi_on=1, tea_epsilon_freq=1)
        b = synth.ragged_batch(p, 5, seed=seed, pf_range=(4, 14), free_range=(0, 300), cube=50.0, radius=8.12,
                               psi_mode="make_mt", thermal=0.05)
        if cutoff_margin(b, b.coords) > 2e-4:
            break
    sizes = np.diff(b.offsets)
    assert sizes.max() > 128 and len(set(sizes.tolist())) > 1, sizes
    o32 = oracle_lib.Oracle("orc", "f32")
    e = make_engine(engine_mod, b)
    eps, beta, ci, rc = e.tea_update()
    assert rc == 0
    ci_o, eps_o = o32.tea_epsilon(b, b.coords)
    eps_t, beta_o, st = o32.tea_beta(b, eps_o)
    assert rel_norm(ci[:, :3], ci_o[:, :3]) < 1e-5
    np.testing.assert_allclose(eps, eps_t, rtol=1e-5)
    np.testing.assert_allclose(beta, beta_o, rtol=1e-5)
    e.close()
    seeds = o32.generate_seeds(b.params.rseed, 2 * b.nbeads)
    xo, _, so, _, st, _, _ = o32.run(b, b.coords, seeds, 0, 1)
    assert st == 0
    for jp in (1, 3):
        e2 = make_engine(engine_mod, b)
        t = e2.tuning()
        e2.set_tuning(t["list_method"], t["step_block"], t["tea_slices"], jp)
        e2.step(0, 1)
        assert np.array_equal(e2.download_rng(), so)
        np.testing.assert_allclose(e2.download_state()[:, :6], xo[:, :6], rtol=0, atol=1e-4)
        e2.close()


@pytest.mark.parametrize("method", [1, 2])
def test_two_bead_trajectory(engine_mod, oracle_lib, method):
    """A ragged batch with a trajectory of a single free dimer beside two
    ordinary ones: lists, forces, energies and one step against the oracle,
    for both rebuild methods."""
    from mt_gb300 import synth
    p = synth.default_params(seed=5)
    trajs = [synth.make_trajectory(6, 20, seed=5, radius=8.12, psi_mode="make_mt", cube=40.0, thermal=0.05),
             synth.make_trajectory(0, 2, seed=7, radius=8.12, psi_mode="make_mt", cube=40.0, thermal=0.05),
             synth.make_trajectory(9, 40, seed=8, radius=8.12, psi_mode="make_mt", cube=40.0, thermal=0.05)]
    b = synth.batch_from_trajectories(p, trajs)
    assert list(np.diff(b.offsets)) == [98, 2, 157]
    o = oracle_lib.Oracle("orc")
    L = o.lists(b, b.coords)
    e = make_engine(engine_mod, b)
    e.set_list_method(method)
    e.rebuild_pairs()
    for k in ("lj", "long", "lat"):
        assert e.list_of_lists(k) == L.as_lists(k), k
    f = e.compute_forces()
    fo = o.forces(b, b.coords, L)
    for c in range(6):
        assert rel_norm(f[:, c], fo[:, c]) < FORCE_RTOL, c
    tot = e.energies()
    eo = o.energies(b, b.coords, L)
    for t in range(b.ntraj):
        sl = slice(int(b.offsets[t]), int(b.offsets[t + 1]))
        np.testing.assert_allclose(tot[t], eo[sl].sum(0), rtol=1e-5, atol=1e-3)
    e.close()
    seeds = o.generate_seeds(p.rseed, 2 * b.nbeads)
    xo, _, so, _, st, _, _ = o.run(b, b.coords, seeds, 0, 1)
    assert st == 0
    e2 = make_engine(engine_mod, b)
    e2.set_list_method(method)
    e2.step(0, 1)
    assert np.array_equal(e2.download_rng(), so)
    np.testing.assert_allclose(e2.download_state()[:, :6], xo[:, :6], rtol=0, atol=5e-5)
    e2.close()


@pytest.mark.parametrize("over", [dict(lj_on=0), dict(ljpairscutoff=5.0)], ids=["lj_off", "lj_cut_5nm"])
@pytest.mark.parametrize("method", [1, 2])
def test_assembly_lists_without_lj_prefilter(engine_mod, oracle_lib, over, method):
    """Assembly lists when the LJ list cannot serve as their prefilter (LJ off,
    or an LJ cutoff below the 6.6 nm reach of the site tests): the rebuild
    runs the site tests itself.  Lists bit-exact, forces within 1e-5."""
    b = system_with_margin(seed=21, **over)
    e = make_engine(engine_mod, b)
    e.set_list_method(method)
    e.rebuild_pairs()
    o = oracle_lib.Oracle("orc")
    L = o.lists(b, b.coords)
    # with LJ off the reference builds no LJ list at all (src/compute_cuda.cu:1141-1144)
    for k in (("lj", "long", "lat") if b.params.lj_on else ("long", "lat")):
        assert e.list_of_lists(k) == L.as_lists(k), k
    if not b.params.lj_on:
        assert all(len(x) == 0 for x in e.list_of_lists("lj"))
    f = e.compute_forces()
    fo = o.forces(b, b.coords, L)
    for c in range(6):
        assert rel_norm(f[:, c], fo[:, c]) < FORCE_RTOL, c
    e.close()


@pytest.mark.parametrize("keep,small", [(False, False), (True, False), (False, True), (True, True)])
def test_persistent_period_equals_per_step_kernels(engine_mod, keep, small):
    """The persistent plain path (one launch per pair-list period, one CTA per
    trajectory with its frames in shared memory) gives the per-step kernels'
    result bit for bit, on an uneven batch with extra and fixed beads, with
    and without stored forces; with trajectories of at most 512 beads (small)
    the pair lists are rebuilt inside the persistent launch, otherwise by the
    list kernels before it."""
    from mt_gb300 import synth
    p = synth.default_params(seed=61)
    trajs = [synth.make_trajectory(14, 120, seed=61, radius=8.12, psi_mode="make_mt", cube=50.0, thermal=0.05,
                                   n_extra_dimers=2),
             synth.make_trajectory(4, 0, seed=62, radius=8.12, psi_mode="make_mt", cube=50.0, thermal=0.05),
             synth.make_trajectory(20, 150, seed=63, radius=8.12, psi_mode="make_mt", cube=50.0, thermal=0.05)
             if small else
             synth.make_trajectory(30, 400, seed=63, radius=8.12, psi_mode="make_mt", cube=60.0, thermal=0.05)]
    b = synth.batch_from_trajectories(p, trajs)
    runs = []
    for persistent in (0, 1):
        e = make_engine(engine_mod, b)
        e.set_keep_forces(keep)
        t = e.tuning()
        e.set_tuning(t["list_method"], t["step_block"], t["tea_slices"], t["tea_jparts"], persistent)
        e.set_kernel_timing(True)
        e.step(0, 35)                      # three periods from graphs + a direct tail
        kt = e.kernel_times()
        assert (kt["step_period"][1] > 0) == bool(persistent)
        if persistent:
            assert (kt["rebuild"][1] == 0) == small, kt["rebuild"]   # lists rebuilt in the launch
        runs.append((e.download_state(forces=True), e.download_rng(), e.lists()))
        e.close()
    (x0, f0), r0, l0 = runs[0]
    (x1, f1), r1, l1 = runs[1]
    assert np.array_equal(x0, x1) and np.array_equal(r0, r1)
    if keep:
        assert np.array_equal(f0, f1)
    for k in ("lj", "long", "lat"):
        assert np.array_equal(l0[k][0], l1[k][0]) and np.array_equal(l0[k][1], l1[k][1])


def test_persistent_rejects_large_trajectories(engine_mod):
    from mt_gb300 import synth
    p = synth.default_params(seed=64)
    b = synth.uniform_batch(p, 1, 120, 2000, seed=64, cube=150.0)     # 3560 beads
    e = make_engine(engine_mod, b)
    t = e.tuning()
    with pytest.raises(engine_mod.MtgError, match="2048"):
        e.set_tuning(t["list_method"], t["step_block"], t["tea_slices"], t["tea_jparts"], 1)
    e.close()


def test_sharded_engine_equals_one_engine(engine_mod):
    """A batch split over engines (here two on the same GPU, independent
    streams, nothing shared) gives the result of one engine of the whole
    batch bit for bit: states, noise streams and energy totals."""
    from mt_gb300 import synth
    p = synth.default_params(seed=71)
    b = synth.ragged_batch(p, 6, seed=71, pf_range=(6, 16), free_range=(0, 200), cube=60.0, radius=8.12,
                           psi_mode="make_mt", thermal=0.05)
    one = make_engine(engine_mod, b)
    one.step(0, 25)
    with engine_mod.ShardedEngine(b, devices=[0, 0]) as sh:
        assert len(sh.engines) == 2
        sh.upload_state(b.coords)
        sh.step(0, 25)
        assert np.array_equal(sh.download_state(), one.download_state())
        assert np.array_equal(sh.download_rng(), one.download_rng())
        np.testing.assert_array_equal(sh.energies(), one.energies())
    one.close()
