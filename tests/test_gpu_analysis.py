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


def _numpy_hist2gofr(nbin, dr, r0, h):
    """pyanalisi/analysis.py:101-105 as the reference evaluates it (numpy)."""
    rs_m = np.arange(nbin) * dr + r0
    rs_p = (np.arange(nbin) + 1) * dr + r0
    vols = 4 * np.pi / 3 * (rs_p ** 3 - rs_m ** 3)
    return h / vols


def _max_rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nz = b != 0
    assert np.array_equal(a[~nz], b[~nz])
    return float(np.max(np.abs(a[nz] - b[nz]) / np.abs(b[nz]))) if nz.any() else 0.0


@pytest.mark.parametrize("case,r0,r1,nbin", [("cellvec_tric", 0.0, 3.0, 30),
                                             ("ortho_wrap", 0.4, 3.3, 57)])
def test_device_normalisation_within_stated_bound(pa, case, r0, r1, nbin):
    """The shell-volume normalisation runs on the GPU in FP64 (correctly
    rounded cubes); its relative difference from the reference's numpy
    hist2gofr on the same buffer is within the bound stated with the result
    (tolerance: that bound, itself below 1e-12 here)."""
    from analisi_gb300 import analysis
    g, traj = _traj(pa, case)
    h = analysis.compute_gofr(traj, r0, r1, nbin, start=0, tmax=2, tskip=3,
                              return_histogram=True)
    assert analysis.last_error_bound == 0.0
    r, bound = analysis.compute_gofr(traj, r0, r1, nbin, start=0, tmax=2, tskip=3,
                                     return_error_bound=True)
    assert bound == analysis.last_error_bound and 0.0 < bound < 1e-12
    want = _numpy_hist2gofr(nbin, (r1 - r0) / nbin, r0, h)
    err = _max_rel(r, want)
    assert err <= bound, (err, bound)


def test_density_normalisation(pa):
    """density=True: each distinct channel also divided by its pair density
    (2 N_a N_b / V, or N_a (N_a - 1) / V for one type), each self channel by
    N_a; against the same formula in numpy, within the stated bound."""
    from analisi_gb300 import analysis
    g, traj = _traj(pa, "ortho_wrap")
    r0, r1, nbin = 0.0, 3.3, 40
    h = analysis.compute_gofr(traj, r0, r1, nbin, start=1, tmax=3, tskip=2,
                              return_histogram=True)
    r, bound = analysis.compute_gofr(traj, r0, r1, nbin, start=1, tmax=3, tskip=2, density=True,
                                     return_error_bound=True)
    nt = int(traj.get_ntypes())
    ids = np.asarray(traj.get_type_ids())
    counts = np.bincount(ids, minlength=nt).astype(float)
    box = np.asarray(traj.get_box_copy())
    stop = traj.get_nloaded_timesteps()
    tm, n_ave = analysis.max_l(1, stop, 3)
    origins = [1 + k * 2 for k in range((n_ave + 1) // 2)]
    V = np.mean([8.0 * box[o, 3] * box[o, 4] * box[o, 5] for o in origins])
    half = nt * (nt + 1) // 2
    fac = np.ones(2 * half)
    for a in range(nt):
        for c in range(a, nt):
            ch = half - (c + 1) * (c + 2) // 2 + a
            fac[ch] = (counts[a] * (counts[a] - 1) if a == c else 2 * counts[a] * counts[c]) / V
            if a == c:
                fac[ch + half] = counts[a]
    want = _numpy_hist2gofr(nbin, (r1 - r0) / nbin, r0, h) / fac[None, :, None]
    err = _max_rel(r, want)
    assert err <= bound < 1e-12, (err, bound)


def test_second_call_on_a_trajectory_copies_no_frames(pa):
    """The frames stay resident between compute_gofr calls on one trajectory:
    the context's host-to-device byte count does not move on the second call;
    another trajectory is uploaded."""
    from analisi_gb300 import analysis
    g, traj = _traj(pa, "ortho_wrap")
    analysis.release_resident()
    a = analysis.compute_gofr(traj, 0.0, 3.3, 40, start=0, tmax=2, tskip=2)
    eng = analysis._resident["engine"]
    before = eng.stats()["h2d_bytes"]
    assert before >= g["positions"].nbytes
    b = analysis.compute_gofr(traj, 0.0, 3.3, 40, start=1, tmax=3, tskip=2, n_segments=2)
    assert analysis._resident["engine"] is eng
    assert eng.stats()["h2d_bytes"] == before
    assert np.all(np.isfinite(a)) and len(b) == 2
    g2, traj2 = _traj(pa, "cellvec_tric")
    analysis.compute_gofr(traj2, 0.0, 3.0, 30, start=0, tmax=2, tskip=3)
    assert analysis._resident["engine"] is not eng
    analysis.release_resident()


def test_device_fold_of_sixteen_partitions_at_16k_atoms(gpu_engine, oracle_mod):
    """The reference's buffer for 16 threads (each partition's count as a
    sequence of incr additions, partitions folded in order), made on the GPU
    from counts of over 10^4 per bin on the 16k-atom workload, equals the
    oracle's fold bit for bit."""
    from analisi_gb300 import workloads
    w = workloads.c2(T=60)
    p = w["params"]
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    got, bound = gpu_engine.gofr(p["rmin"], p["rmax"], p["nbin"], 3, 7, 1, 21, [0, 5],
                                 norm="buffer", nparts=16)
    assert bound == 0.0
    for k, primo in enumerate([0, 5]):
        per = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                      p["rmin"], p["rmax"], p["nbin"], 3, 16, 7, 1, 21, primo,
                                      per_thread=True)
        want = oracle_mod.fold_buffer(per, oracle_mod.incr(21, 7))
        assert per.max() > 10000
        assert np.array_equal(got[k].view(np.uint64), want.view(np.uint64))


def test_max_l_matches_reference_rules():
    from analisi_gb300 import analysis
    assert analysis.max_l(0, 100, 0) == (50, 50)
    assert analysis.max_l(10, 20, 15) == (9, 1)
    with pytest.raises(RuntimeError):
        analysis.max_l(5, 5, 1)
