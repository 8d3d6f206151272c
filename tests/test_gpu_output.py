"""Stride-step outputs through pinned buffers and the writer thread: the DCD
files equal, byte for byte, what the reference's writer (restated in
oracle/dcd_oracle.py, itself checked against src/dcdio.cpp) makes of the
states at those steps, and the energy lines are the reference's."""
import numpy as np
import pytest

from helpers import small_system
from oracle import dcd_oracle as D

pytestmark = pytest.mark.gpu


def test_async_dcd_and_energy_output(engine_mod, tmp_path, capfd):
    b = small_system(seed=51, ntr=3)
    stride, frames = 5, 4
    xyz = [str(tmp_path / f"xyz{t}.dcd") for t in range(b.ntraj)]
    ang = [str(tmp_path / f"ang{t}.dcd") for t in range(b.ntraj)]
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.output_open(xyz, ang, nfile=frames, npriv=1, nsavc=stride, delta=100.0, remark2="REMARKS TEST")
    for k in range(frames):
        e.step(k * stride, stride)
        e.output_frame((k + 1) * stride, frame=True, energies=True)
    assert e.output_flush() == frames
    e.output_close()
    e.close()
    printed = [ln for ln in capfd.readouterr().out.splitlines() if ln.startswith("Energies[")]

    # the same run, downloaded synchronously at every stride step
    ref = engine_mod.Engine(b)
    ref.upload_state(b.coords)
    states, lines = [], []
    for k in range(frames):
        ref.step(k * stride, stride)
        states.append(ref.download_state())
        for t, u in enumerate(ref.energies()):
            lines.append(f"Energies[{t}]:\t" + "\t".join(f"{v:f}" for v in u))
    ref.close()
    expect = D.trajectory_files(states, b.offsets, frames, 1, stride, 100.0, "REMARKS TEST")
    for t in range(b.ntraj):
        assert open(xyz[t], "rb").read() == expect[t][0]
        assert open(ang[t], "rb").read() == expect[t][1]
    assert printed == lines


def test_dcd_frames_read_back_for_reanalysis(engine_mod, tmp_path):
    """The written frames read back (mt_gb300.dcd) as the states of those
    steps, and their energies re-evaluated on the GPU match the run's."""
    from mt_gb300 import dcd
    b = small_system(seed=52, ntr=2)
    stride, frames = 4, 3
    xyz = [str(tmp_path / f"x{t}.dcd") for t in range(b.ntraj)]
    ang = [str(tmp_path / f"a{t}.dcd") for t in range(b.ntraj)]
    e = engine_mod.Engine(b)
    e.upload_state(b.coords)
    e.output_open(xyz, ang, frames, 1, stride, 100.0, "REMARKS TEST", energy_path=str(tmp_path / "en.txt"))
    states, energies = [], []
    for k in range(frames):
        e.step(k * stride, stride)
        e.output_frame((k + 1) * stride)
        states.append(e.download_state())
        e.rebuild_pairs()
        energies.append(e.energies())
    e.output_close()
    back = list(dcd.read_batch(xyz, ang))
    assert len(back) == frames
    for k in range(frames):
        np.testing.assert_array_equal(back[k][:, :6], states[k][:, :6])
    again = dcd.analyse(e, xyz, ang)
    np.testing.assert_allclose(again, np.array(energies), rtol=1e-12, atol=1e-9)
    e.close()
