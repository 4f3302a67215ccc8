"""g(r,t) over the reference's memory-mapped trajectory (`Gofrt_lammps` over
`Traj`, pyanalisi/src/pyanalisi.cpp:376-418,534-535) and over frames streamed
through the device under a memory budget (the reference bounds its memory
with a window of frames, lib/src/trajectory.cpp:349-384,450-690).  Results
must equal, bit for bit, the same calculation on the whole trajectory held
resident, and the oracle's counts."""
import numpy as np
import pytest

import lammps_writer
from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pa(built_engine):
    from analisi_gb300 import build
    build.build_host()
    import analisi_gb300
    return analisi_gb300.load_pyanalisi()


def _written(tmp_path, w):
    p = str(tmp_path / "traj.bin")
    lammps_writer.write(p, w["positions"], w["types"], w["box_lammps"], w["triclinic"], nchunk=2)
    return p


@pytest.mark.parametrize("wrap", [False, True])
def test_gofrt_lammps_equals_whole_trajectory_and_oracle(pa, oracle_mod, tmp_path, wrap):
    w = workloads.small_case(81, 900, 40, 20.0, 0.15, [600, 300], rmin=0.0, rmax=6.0, nbin=60)
    p = _written(tmp_path, w)
    d = pa.read_lammps_binary(p)
    whole = pa.Trajectory(d["positions"], d["velocities"], d["types"], d["boxes"],
                          pa.BoxFormat.LammpsOrtho, wrap, False)
    traj = pa.Traj(p)
    traj.setWrapPbc(wrap)
    traj.setAccessWindowSize(12)  # shorter than a calculation needs: grown on demand
    traj.setAccessStart(0)
    g_w = pa.Gofrt_lammps(traj, 0.0, 6.0, 60, 5, 3, 2, 1, False)
    g_a = pa.Gofrt(whole, 0.0, 6.0, 60, 5, 3, 2, 1, False)
    for g in (g_w, g_a):
        g.reset(16)
    for primo in (0, 7, 19):  # windows moved on demand
        g_w.calculate(primo)
        g_a.calculate(primo)
        a, b = np.array(g_w, copy=True), np.array(g_a, copy=True)
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
        counts = oracle_mod.gofrt_counts(whole.get_positions_copy(), whole.get_box_copy(),
                                         whole.get_type_ids(), whole.get_ntypes(), 0.0, 6.0, 60,
                                         5, 3, 2, 1, 16, primo)
        assert np.array_equal(np.rint(a * 8).astype(np.uint64), counts)  # incr = 1/8
    assert traj.get_current_timestep() == 19
    with pytest.raises(RuntimeError):
        g_w.calculate(30)  # frames 30 .. 49 are past the end of the 40-frame file


@pytest.mark.parametrize("budget_frames", [6, 9, 25])
def test_streamed_counts_equal_resident_counts(built_engine, oracle_mod, budget_frames):
    """Origins streamed in chunks whose frames fit a device budget (6 frames:
    one origin per chunk with its 4 lags) give gofr_run's counts."""
    from analisi_gb300 import engine
    w = workloads.small_case(82, 2000, 40, 27.0, 0.2, [1200, 800], rmin=0.0, rmax=6.0, nbin=50)
    per_frame = ((2000 + 15) // 16 * 16) * 64 + 512
    with engine.Engine(0) as e:
        e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        for nparts, kernel in ((1, "auto"), (3, "auto"), (1, "cellw"), (1, "f64")):
            args = (0.0, 6.0, 50, 5, 3, 1, 20, 2)
            want = e.run(*args, kernel=kernel, nparts=nparts)
            e2 = engine.Engine(0)
            got = e2.run_streamed(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                  budget_frames * per_frame, *args, kernel=kernel, nparts=nparts)
            e2.close()
            np.testing.assert_array_equal(got, want)
            e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"], 0.0,
                                  6.0, 50, 5, 8, 3, 1, 20, 2)
    np.testing.assert_array_equal(want, ref)


def test_streamed_budget_too_small_is_refused(built_engine):
    from analisi_gb300 import engine
    w = workloads.small_case(83, 200, 20, 12.0, 0.2, [200], rmin=0.0, rmax=5.0, nbin=20)
    with engine.Engine(0) as e:
        with pytest.raises(engine.GofrError) as err:
            e.run_streamed(w["positions"], w["boxes"], w["type_ids"], w["ntypes"], 1000, 0.0,
                           5.0, 20, 5, 1, 1, 10, 0)
        assert err.value.code == -7


def test_gofrt_device_budget_streams_with_identical_result(pa, monkeypatch):
    """The drop-in Gofrt with a device budget far below its trajectory streams
    the frames in chunks of origins; its buffer equals the resident run's."""
    w = workloads.small_case(84, 1500, 60, 24.0, 0.15, [1000, 500], rmin=0.0, rmax=5.0, nbin=40)
    traj = pa.Trajectory(w["positions"], np.zeros_like(w["positions"]), w["types"],
                         w["box_lammps"], pa.BoxFormat.LammpsOrtho, False, False)
    g_a = pa.Gofrt(traj, 0.0, 5.0, 40, 6, 2, 4, 1, False)
    g_s = pa.Gofrt(traj, 0.0, 5.0, 40, 6, 2, 4, 1, False)
    g_s.set_device_budget(12 * 1500 * 64)  # about 12 frames of 60
    for g in (g_a, g_s):
        g.reset(40)
        g.calculate(3)
    a, b = np.array(g_a, copy=True), np.array(g_s, copy=True)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
