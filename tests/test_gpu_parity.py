"""GPU parity: exact counts of the CUDA kernels against the oracle (the C
restatement of the reference's Gofrt, oracle/gofr_oracle.c) on seeded inputs.

Mirrors the reference's own gofr tests (tests/test_gofrt.py: Gofrt(...),
reset(n), calculate(primo), compare the whole result buffer) and the C++
regression (tests/src/test_lammps2020.cpp:27-48: several thread counts, tmax
and primo), with integer counts compared bit for bit.
"""
import numpy as np
import pytest

from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu


def _oracle_counts(oracle_mod, w, nthreads=1, per_thread=False):
    p = w["params"]
    pos = w.get("internal_positions", w["positions"])
    return oracle_mod.gofrt_counts(pos, w["boxes"], w["type_ids"], w["ntypes"], p["rmin"],
                                   p["rmax"], p["nbin"], p["tmax"], nthreads, p["skip"],
                                   p["every"], p["ntimesteps"], p["primo"], tric=w["triclinic"],
                                   per_thread=per_thread)


def _gpu_counts(eng, w, kernel="auto", nparts=1):
    p = w["params"]
    pos = w.get("internal_positions", w["positions"])
    eng.set_frames(pos, w["boxes"], w["type_ids"], w["ntypes"], triclinic=w["triclinic"])
    return eng.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                   p["ntimesteps"], p["primo"], kernel=kernel, nparts=nparts)


CASES = [
    # seed, N, T, L, sigma, counts, tric, wrap_into_cell, params
    (11, 64, 40, 7.0, 0.3, [32, 32], False, False,
     dict(rmin=0.0, rmax=3.4, nbin=40, tmax=6, skip=4, every=1, ntimesteps=30, primo=2)),
    (12, 100, 30, 9.0, 0.2, [50, 30, 20], False, True,
     dict(rmin=0.5, rmax=4.4, nbin=33, tmax=0, skip=3, every=2, ntimesteps=14, primo=1)),
    (13, 80, 30, 8.0, 0.25, [80], True, True,
     dict(rmin=0.0, rmax=3.9, nbin=50, tmax=5, skip=7, every=1, ntimesteps=20, primo=0)),
    (14, 600, 12, 18.0, 0.1, [300, 200, 100], False, False,
     dict(rmin=0.0, rmax=6.0, nbin=120, tmax=4, skip=2, every=1, ntimesteps=8, primo=0)),
    (15, 700, 12, 20.0, 0.1, [350, 350], True, True,
     dict(rmin=0.3, rmax=7.0, nbin=97, tmax=3, skip=3, every=1, ntimesteps=9, primo=0)),
    # small box: rmax > l/2, the wrap-decision check is on
    (16, 50, 20, 5.0, 0.3, [25, 25], False, False,
     dict(rmin=0.0, rmax=4.0, nbin=60, tmax=4, skip=2, every=1, ntimesteps=15, primo=1)),
    (17, 60, 20, 6.0, 0.3, [20, 20, 20], True, True,
     dict(rmin=0.0, rmax=5.0, nbin=45, tmax=4, skip=3, every=2, ntimesteps=15, primo=0)),
    # spans several shared-memory tiles and first-atom tiles
    (18, 2500, 6, 30.0, 0.1, [1000, 1500], False, False,
     dict(rmin=0.0, rmax=9.0, nbin=200, tmax=2, skip=2, every=1, ntimesteps=4, primo=0)),
]


@pytest.mark.parametrize("case", CASES, ids=[f"seed{c[0]}" for c in CASES])
@pytest.mark.parametrize("kernel", ["auto", "f64"])
def test_counts_match_oracle(gpu_engine, oracle_mod, case, kernel):
    seed, N, T, L, sigma, counts, tric, wrap, params = case
    w = workloads.small_case(seed, N, T, L, sigma, counts, tric=tric, wrap_into_cell=wrap,
                             **params)
    ref = _oracle_counts(oracle_mod, w)
    got = _gpu_counts(gpu_engine, w, kernel=kernel)
    assert got.shape == ref.shape
    assert got.sum() > 0
    np.testing.assert_array_equal(got, ref)
    st = gpu_engine.stats()
    if kernel == "f64":
        assert st["kernel_used"] == 2
    else:
        assert st["kernel_used"] == 1


def test_c1_config_exact(gpu_engine, oracle_mod):
    """Config 1 (N=1000, 2 types, 3.6e8 pairs): full parity."""
    w = workloads.c1()
    ref = _oracle_counts(oracle_mod, w, nthreads=8)
    got = _gpu_counts(gpu_engine, w)
    np.testing.assert_array_equal(got, ref)
    assert int(got.sum()) == int(ref.sum())


def test_partition_counts_and_exact_buffer(gpu_engine, oracle_mod):
    """nparts = reference threads: per-partition counts rebuild the reference's
    double buffer bit for bit (gofrt.cpp:118,128-132)."""
    from analisi_gb300 import engine
    seed, N, T, L, sigma, counts, tric, wrap, params = CASES[3]
    w = workloads.small_case(seed, N, T, L, sigma, counts, tric=tric, wrap_into_cell=wrap,
                             **params)
    ref = _oracle_counts(oracle_mod, w, nthreads=3, per_thread=True)
    got = _gpu_counts(gpu_engine, w, nparts=3)
    np.testing.assert_array_equal(got, ref)
    p = w["params"]
    buf = engine.counts_to_buffer(got, p["ntimesteps"], p["skip"], nparts=3)
    assert buf.shape == got.shape[1:]
    obuf = oracle_mod.fold_buffer(ref, oracle_mod.incr(p["ntimesteps"], p["skip"]))
    assert np.array_equal(buf.view(np.uint64), obuf.view(np.uint64))


def test_too_short_raises(gpu_engine):
    from analisi_gb300 import engine
    w = workloads.small_case(3, 20, 10, 6.0, 0.1, [20], rmin=0.0, rmax=2.0, nbin=10)
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    with pytest.raises(engine.TrajectoryTooShort):
        gpu_engine.run(0.0, 2.0, 10, tmax=5, skip=1, every=1, ntimesteps=7, primo=0)
