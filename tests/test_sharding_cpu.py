"""The split of a batch over several GPUs (ShardedEngine, the replacement of
the reference's MPI replicas, src/main.cpp:27-48): contiguous groups of
trajectories, every trajectory in exactly one group, bead counts balanced;
sub-batches keep each trajectory's data."""
import numpy as np

from mt_gb300 import engine, synth


def test_split_covers_every_trajectory_once_and_balances_beads():
    rng = np.random.default_rng(1)
    sizes = rng.integers(100, 3600, size=1024)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for parts in (1, 2, 3, 4, 8):
        sp = engine.split_by_beads(off, parts)
        assert len(sp) == parts and sp[0][0] == 0 and sp[-1][1] == 1024
        assert all(a[1] == b[0] for a, b in zip(sp, sp[1:]))          # contiguous, no overlap
        loads = [int(off[t1] - off[t0]) for t0, t1 in sp]
        assert sum(loads) == int(off[-1])
        assert max(loads) - min(loads) <= 2 * sizes.max(), loads       # within a trajectory or two


def test_split_with_fewer_trajectories_than_parts():
    off = np.array([0, 10, 30])
    sp = engine.split_by_beads(off, 4)
    assert sp[0][0] == 0 and sp[-1][1] == 2
    assert sorted(t for t0, t1 in sp for t in range(t0, t1)) == [0, 1]


def test_sub_batch_keeps_trajectory_data():
    p = synth.default_params(seed=3)
    b = synth.ragged_batch(p, 5, seed=3, pf_range=(4, 10), free_range=(0, 40), cube=50.0, radius=8.12)
    s = synth.sub_batch(b, 1, 4)
    b0, b1 = int(b.offsets[1]), int(b.offsets[4])
    assert s.ntraj == 3 and s.nbeads == b1 - b0
    assert np.array_equal(np.diff(s.offsets), np.diff(b.offsets[1:5]))
    assert np.array_equal(s.coords, b.coords[b0:b1]) and np.array_equal(s.harmonic, b.harmonic[b0:b1])
    assert np.array_equal(s.zs, b.zs[1:4])
