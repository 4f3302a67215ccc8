"""The reference's memory-mapped trajectory (`Traj`,
pyanalisi/src/pyanalisi.cpp:376-418; lib/src/trajectory.cpp): a binary file
mapped into memory, a window of frames decoded at a time.  Host checks (no
GPU): every window equals the same frames of the whole file read at once and
preprocessed by the numpy-input Trajectory, wrapped or not, positions and
velocities through the buffer protocol, and the reference's return codes."""
import numpy as np
import pytest

import lammps_writer


@pytest.fixture(scope="module")
def pa(built_engine):
    from analisi_gb300 import build
    build.build_host()
    import analisi_gb300
    return analisi_gb300.load_pyanalisi()


def _file(tmp_path, triclinic, T=20, N=37):
    rng = np.random.default_rng(71 + triclinic)
    pos = rng.uniform(-4, 12, (T, N, 3))
    types = rng.integers(1, 4, N).astype(np.int32)
    row = [0, 8.0, -1, 7.5, 0.5, 9.0] + ([1.0, 0.5, -0.3] if triclinic else [])
    boxes = np.tile(row, (T, 1)).astype(float)
    boxes[:, 1] += 0.01 * np.arange(T)  # a box that changes from frame to frame
    p = str(tmp_path / f"w{int(triclinic)}.bin")
    lammps_writer.write(p, pos, types, boxes, triclinic, nchunk=2, perm=rng.permutation(N))
    return p


@pytest.mark.parametrize("triclinic", [False, True])
@pytest.mark.parametrize("wrap", [False, True])
def test_windows_equal_the_whole_file(pa, tmp_path, triclinic, wrap):
    p = _file(tmp_path, triclinic)
    d = pa.read_lammps_binary(p)
    fmt = pa.BoxFormat.LammpsTriclinic if triclinic else pa.BoxFormat.LammpsOrtho
    whole = pa.Trajectory(d["positions"], d["velocities"], d["types"], d["boxes"], fmt, wrap,
                          False)
    t = pa.Traj(p)
    t.setWrapPbc(wrap)
    assert t.getNtimesteps() == 20 and t.get_natoms() == 37
    assert t.get_ntypes() == whole.get_ntypes()
    assert t.setAccessWindowSize(5) == 1
    for start in (0, 3, 15):
        assert t.setAccessStart(start) == 1
        assert t.get_current_timestep() == start and t.get_nloaded_timesteps() == 5
        np.testing.assert_array_equal(t.get_positions_copy(),
                                      whole.get_positions_copy()[start:start + 5])
        np.testing.assert_array_equal(t.get_box_copy(), whole.get_box_copy()[start:start + 5])
        assert t.serving_pos()
        np.testing.assert_array_equal(np.array(t), whole.get_positions_copy()[start:start + 5])
        t.toggle_pos_vel()
        np.testing.assert_array_equal(np.array(t), whole.get_velocities_copy()[start:start + 5])
        t.toggle_pos_vel()
    np.testing.assert_array_equal(t.get_type_ids(), whole.get_type_ids())
    assert list(t.get_lammps_timesteps()) == list(d["timesteps"])


def test_window_return_codes(pa, tmp_path):
    t = pa.Traj(_file(tmp_path, False))
    with pytest.raises(RuntimeError):
        t.get_positions_copy()  # nothing loaded yet
    assert t.setAccessWindowSize(0) == 0
    assert t.setAccessWindowSize(8) == 1
    assert t.setAccessStart(13) == 2  # the window would pass the end of the file
    assert t.setAccessStart(12) == 1
    with pytest.raises(RuntimeError):
        pa.Traj(str(tmp_path / "missing.bin"))
    assert pa.has_mmap()
