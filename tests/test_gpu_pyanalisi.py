"""The drop-in Python API end to end on the GPU, written like the reference's
tests/test_gofrt.py: pyanalisi.Gofrt(traj, rmin, rmax, nbin, tmax, nthreads,
skip, every, debug), reset(n), calculate(primo), np.array(gofr) -- compared
bit for bit with the buffers the reference itself produced (tests/golden/)."""
import numpy as np
import pytest

import golden_util as gu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pa(built_engine):
    from analisi_gb300 import build
    build.build_host()
    import analisi_gb300
    return analisi_gb300.load_pyanalisi()


@pytest.mark.parametrize("name", gu.names())
def test_gofr_buffer_bit_identical(pa, name):
    g = gu.load(name)
    m = g["meta"]
    traj = pa.Trajectory(g["positions"], np.zeros_like(g["positions"]), g["types"], g["box"],
                         getattr(pa.BoxFormat, m["box_format"]), m["wrap"], False)
    gofr = pa.Gofrt(traj, m["rmin"], m["rmax"], m["nbin"], m["tmax"], m["nthreads"], m["skip"],
                    m["every"], False)
    gofr.reset(m["ntimesteps"])
    gofr.calculate(m["primo"])
    gr = np.array(gofr, copy=True)
    ref = g["ref_buffer"]
    assert gr.shape == ref.shape
    assert np.array_equal(gr.view(np.uint64), ref.view(np.uint64))
    assert gofr.get_columns_description() == m["columns"]
    st = gofr.last_stats()
    assert st["pairs"] > 0


def test_plain_fp64_kernel_same_buffer(pa):
    g = gu.load("ortho_wrap")
    m = g["meta"]
    traj = pa.Trajectory(g["positions"], np.zeros_like(g["positions"]), g["types"], g["box"],
                         pa.BoxFormat.LammpsOrtho, m["wrap"], False)
    gofr = pa.Gofrt(traj, m["rmin"], m["rmax"], m["nbin"], m["tmax"], m["nthreads"], m["skip"],
                    m["every"], False)
    gofr.set_kernel(2)
    gofr.reset(m["ntimesteps"])
    gofr.calculate(m["primo"])
    assert gofr.last_stats()["kernel_used"] == 2
    assert np.array_equal(np.array(gofr).view(np.uint64), g["ref_buffer"].view(np.uint64))


def test_too_short_raises_runtime_error(pa):
    g = gu.load("ortho_lammps")
    traj = pa.Trajectory(g["positions"], np.zeros_like(g["positions"]), g["types"], g["box"],
                         pa.BoxFormat.LammpsOrtho, False, False)
    gofr = pa.Gofrt(traj, 0.0, 3.0, 10, 0, 1, 1, 1, False)
    gofr.reset(g["positions"].shape[0])
    with pytest.raises(RuntimeError, match="trajectory is too short"):
        gofr.calculate(0)
