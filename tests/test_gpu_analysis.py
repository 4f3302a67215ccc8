"""Python conveniences (analisi_gb300.analysis, restating
pyanalisi/analysis.py:77-145): compute_gofr, single and segmented (all
segments in one launch), equals Gofrt.calculate per segment through the
drop-in module -- which is pinned bit for bit to the reference -- and the
oracle's counts."""
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


def _traj(pa, name):
    g = gu.load(name)
    m = g["meta"]
    return g, pa.Trajectory(g["positions"], np.zeros_like(g["positions"]), g["types"], g["box"],
                            getattr(pa.BoxFormat, m["box_format"]), m["wrap"], False)


@pytest.mark.parametrize("nthreads", [1, 3])
@pytest.mark.parametrize("n_segments", [1, 3])
def test_compute_gofr_matches_gofrt_per_segment(pa, nthreads, n_segments):
    from analisi_gb300 import analysis
    g, traj = _traj(pa, "ortho_wrap")
    startr, endr, nbin, tskip, tmax = 0.0, 3.3, 40, 2, 4
    stop = traj.get_nloaded_timesteps()
    res = analysis.compute_gofr(traj, startr, endr, nbin, start=1, stop=stop, tmax=tmax,
                                tskip=tskip, n_segments=n_segments, nthreads=nthreads,
                                return_histogram=True)
    tm, n_ave = analysis.max_l(1, stop, tmax)
    gofr = pa.Gofrt(traj, startr, endr, nbin, tm, nthreads, tskip, 1, False)
    if n_segments == 1:
        gofr.reset(n_ave)
        gofr.calculate(1)
        want = [np.array(gofr, copy=True)]
        res = [res]
    else:
        seg = max(1, n_ave // n_segments)
        gofr.reset(seg)
        want = []
        for i in range(0, min(seg * n_segments, n_ave), seg):
            gofr.calculate(1 + i)
            want.append(np.array(gofr, copy=True))
    assert len(res) == len(want)
    for a, b in zip(res, want):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_hist2gofr_normalisation(pa):
    from analisi_gb300 import analysis
    g, traj = _traj(pa, "cellvec_tric")
    r = analysis.compute_gofr(traj, 0.0, 3.0, 30, start=0, tmax=2, tskip=3)
    h = analysis.compute_gofr(traj, 0.0, 3.0, 30, start=0, tmax=2, tskip=3,
                              return_histogram=True)
    dr = 3.0 / 30
    vols = 4 * np.pi / 3 * (((np.arange(30) + 1) * dr) ** 3 - (np.arange(30) * dr) ** 3)
    assert np.array_equal(r, h / vols)


def test_max_l_matches_reference_rules():
    from analisi_gb300 import analysis
    assert analysis.max_l(0, 100, 0) == (50, 50)
    assert analysis.max_l(10, 20, 15) == (9, 1)
    with pytest.raises(RuntimeError):
        analysis.max_l(5, 5, 1)
