"""Oracle parity at the full sizes of the five Gofrt workloads.

The small-case parity tests pin every kernel on inputs the oracle finishes in
milliseconds; these run the same comparison on the workloads the benchmark
measures -- the 16k-atom cubic box, the 32k-atom triclinic cell, members of
the 64-trajectory batch and the 131k-atom box -- with the frames of the whole
trajectory resident, the engine's default plan (the cell-list kernel where it
takes it, with its own certified windows) and the all-pairs FP32 and plain
FP64 kernels, against the oracle (the C restatement of
lib/src/gofrt.cpp:96-122) on (origin, lag) samples it finishes in seconds.

A sample of lags {0, L} at origin o is one calculate(o) with
reset(L + 1), tmax = L + 1, skip = L + 1 (one origin) and every = L, the
reference's own lag grid (lib/include/calculatemultithread.h:50-78).  Every
bin must match exactly.
"""
import os

import numpy as np
import pytest

from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _sample_params(w, primo, lag):
    """calculate(primo) over lags {0, lag} (every = lag) at one origin."""
    p = dict(w["params"])
    n = lag + 1
    p.update(tmax=n, skip=n, every=max(lag, 1), ntimesteps=n, primo=primo)
    return p


def _oracle(oracle_mod, w, p):
    return oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                   p["rmin"], p["rmax"], p["nbin"], p["tmax"], THREADS, p["skip"],
                                   p["every"], p["ntimesteps"], p["primo"], tric=w["triclinic"])


def _gpu(eng, p, kernel):
    c = eng.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                p["ntimesteps"], p["primo"], kernel=kernel)
    return c, eng.stats()


def _check_samples(eng, oracle_mod, w, samples, kernels):
    """Every (primo, lag) sample through every kernel against the oracle;
    returns the kernels the engine reported per requested kernel."""
    used = {k: set() for k in kernels}
    for primo, lag in samples:
        p = _sample_params(w, primo, lag)
        ref = _oracle(oracle_mod, w, p)
        assert ref.sum() > 0
        for k in kernels:
            got, st = _gpu(eng, p, k)
            used[k].add(st["kernel_used"])
            assert got.shape == ref.shape
            bad = int((got != ref).sum())
            assert bad == 0, f"{w['name']} primo={primo} lag={lag} kernel={k}: {bad} bins differ"
    return used


def test_c2_16k_atoms_default_plan_all_pairs_and_fp64(gpu_engine, oracle_mod):
    """16384 atoms (16352/16/16), L=54.72, 400 bins on [0, 12]: origins 0 and
    1000, lags {0, 1, 100, 199}, through the default plan (the warp-streamed
    cell-list kernel the benchmark times), the block cell-list kernel, the
    all-pairs FP32 kernel and plain FP64."""
    w = workloads.c2()
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    samples = [(o, lag) for o in (0, 1000) for lag in (1, 100, 199)]
    used = _check_samples(gpu_engine, oracle_mod, w, samples, ["auto", "cell", "cellw", "f32",
                                                               "f64"])
    assert used == {"auto": {5}, "cell": {3}, "cellw": {5}, "f32": {1}, "f64": {2}}


def test_c3_32k_atoms_triclinic(gpu_engine, oracle_mod):
    """32768 atoms in the triclinic cell a=(L,0,0), b=(0.3L,L,0),
    c=(0.2L,0.1L,L), L=70, 500 bins on [0, 15]: origins 0 and 500, lags
    {0, 1, 50}, through the default plan (the warp-streamed cell-list kernel
    on tilted cells), the all-pairs FP32 kernel and plain FP64."""
    w = workloads.c3()
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"], triclinic=True)
    samples = [(o, lag) for o in (0, 500) for lag in (1, 50)]
    used = _check_samples(gpu_engine, oracle_mod, w, samples, ["auto", "cellw", "f32", "f64"])
    assert used == {"auto": {5}, "cellw": {5}, "f32": {1}, "f64": {2}}


def test_c5_131k_atoms_cells_against_fp64_all_pairs(gpu_engine, oracle_mod):
    """131072 atoms (4 x 25 %), L=109.47, 250 bins on [0, 10]: origin 0, lags
    {0, 24, 48} through both cell-list kernels, the default plan and the
    all-pairs FP64 kernel, all against the oracle."""
    w = workloads.c5()
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    p = dict(w["params"])
    p.update(tmax=49, skip=49, every=24, ntimesteps=49, primo=0)
    ref = _oracle(oracle_mod, w, p)
    assert ref.sum() > 0
    cell, st = _gpu(gpu_engine, p, "cell")
    assert st["kernel_used"] == 3 and st["evaluated"] < st["pairs"] // 10
    np.testing.assert_array_equal(cell, ref)
    cellw, st = _gpu(gpu_engine, p, "cellw")
    assert st["kernel_used"] == 5 and st["evaluated"] < st["pairs"] // 20
    np.testing.assert_array_equal(cellw, ref)
    auto, st = _gpu(gpu_engine, p, "auto")
    assert st["kernel_used"] == 5
    np.testing.assert_array_equal(auto, ref)
    f64, st = _gpu(gpu_engine, p, "f64")
    assert st["kernel_used"] == 2
    np.testing.assert_array_equal(f64, ref)


# members of the 64-trajectory batch: the smallest (N=265, box edge < 2 rmax:
# the per-pair wrap check), 519 atoms in 4 types, 3669 atoms (all-pairs) and
# 6520 atoms in 4 types (the cell-list launch)
C4_MEMBERS = (27, 35, 4, 48)


def test_c4_batch_members_one_graph(built_engine, oracle_mod):
    """Four members of the uneven batch in one graph-captured batch (persistent
    all-pairs work queue + multi-trajectory cell-list launch), replayed twice,
    each member's counts against the oracle.  The two small members run their
    full calculation (every origin of stride 5, lags up to min(100, T/2)); the
    two large ones 2 origins (stride 50) x every 7th lag."""
    from analisi_gb300 import engine
    mem = [workloads.c4_member(k) for k in C4_MEMBERS]
    trajs, refs = [], []
    for m in mem:
        p = dict(m["params"])
        if m["positions"].shape[1] > 1000:
            p.update(ntimesteps=100, skip=50, every=7)
        refs.append(oracle_mod.gofrt_counts(m["positions"], m["boxes"], m["type_ids"],
                                            m["ntypes"], p["rmin"], p["rmax"], p["nbin"],
                                            p["tmax"], THREADS, p["skip"], p["every"],
                                            p["ntimesteps"], p["primo"]))
        trajs.append(dict(positions=m["positions"], boxes=m["boxes"], type_ids=m["type_ids"],
                          ntypes=m["ntypes"],
                          params=engine.make_params(p["rmin"], p["rmax"], p["nbin"], p["tmax"],
                                                    p["skip"], p["every"], p["ntimesteps"],
                                                    p["primo"])))
    with engine.Engine(0) as e:
        e.batch_set(trajs)
        for rep in range(2):
            outs = e.batch_run(use_graph=True)
            st = e.stats()
            assert st["evaluated"] < st["pairs"]  # the large member ran with cell lists
            for k, (got, ref) in enumerate(zip(outs, refs)):
                assert got.shape == ref.shape
                bad = int((got != ref).sum())
                assert bad == 0, f"member {C4_MEMBERS[k]} replay {rep}: {bad} bins differ"
