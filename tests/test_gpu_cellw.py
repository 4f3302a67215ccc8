"""Warp-streamed cell-list kernel (GOFR_KERNEL_CELL_WARP): each warp streams
the neighbourhood of its own small block of cells through 1-D bulk copies.
Counts must equal the oracle's for every configuration: reach 1, 2 and 3,
warp blocks whose neighbourhood wraps the box on every axis, several batches
of first atoms per block, chunks packed from several rows, shifted and non-cubic
boxes, unwrapped coordinates far outside the box, and thousands of FP64
rechecks (a warp's recheck queue overflowing)."""
import numpy as np
import pytest

from analisi_gb300 import workloads

from test_gpu_cells import CASES, copies_on_thresholds

pytestmark = pytest.mark.gpu


def _run(eng, w, kernel):
    p = w["params"]
    eng.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    c = eng.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                p["ntimesteps"], p["primo"], kernel=kernel)
    return c, eng.stats()


def _ref(oracle_mod, w):
    p = w["params"]
    return oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                   p["rmin"], p["rmax"], p["nbin"], p["tmax"], 8, p["skip"],
                                   p["every"], p["ntimesteps"], p["primo"])


# "reach,r,wx,wy,wz" through ANALISI_GB300_CELLW_PLAN (None: the planner's
# choice; r is the 4 records a lane holds); blocks of 2 x 2 x 1 and 2 x 2 x 2
# cells of reach 1 hold more than one batch of 64 first atoms
PLANS = [None, "1,4,1,1,1", "1,4,2,2,1", "2,4,1,2,2", "2,4,3,1,1", "2,4,2,2,2", "3,4,2,2,2",
         "1,4,2,2,2"]


@pytest.mark.parametrize("plan", PLANS, ids=[str(p) for p in PLANS])
@pytest.mark.parametrize("case", CASES, ids=[str(c[0]) for c in CASES])
def test_cellw_matches_oracle(gpu_engine, oracle_mod, case, plan, monkeypatch):
    if plan is None:
        monkeypatch.delenv("ANALISI_GB300_CELLW_PLAN", raising=False)
    else:
        monkeypatch.setenv("ANALISI_GB300_CELLW_PLAN", plan)
    seed, N, T, L, sigma, counts, params = case
    w = workloads.small_case(seed, N, T, L, sigma, counts, **params)
    if seed == 62:  # shifted, non-cubic box
        w["boxes"] = w["boxes"].copy()
        w["boxes"][:, 0] -= 3.0
        w["boxes"][:, 4] *= 1.08
    ref = _ref(oracle_mod, w)
    got, st = _run(gpu_engine, w, "cellw")
    assert st["kernel_used"] == 5
    assert st["evaluated"] <= st["pairs"]
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("plan", [None, "1,4,1,1,1", "2,4,2,1,2"])
def test_cellw_far_unwrapped_coordinates(gpu_engine, oracle_mod, plan, monkeypatch):
    """Atoms several box lengths outside a box that is not at the origin."""
    if plan is None:
        monkeypatch.delenv("ANALISI_GB300_CELLW_PLAN", raising=False)
    else:
        monkeypatch.setenv("ANALISI_GB300_CELLW_PLAN", plan)
    w = workloads.small_case(65, 2400, 7, 26.0, 0.4, [1500, 900], rmin=0.3, rmax=5.0, nbin=45,
                             tmax=3, skip=2, every=1, ntimesteps=4, primo=0)
    rng = np.random.default_rng(650)
    L = 26.0
    w["positions"] = w["positions"] + L * rng.integers(-4, 5, size=(1, 2400, 3))
    w["boxes"] = w["boxes"].copy()
    w["boxes"][:, 0:3] += np.array([-7.5, 3.25, 11.0])
    w["positions"] = w["positions"] + np.array([-7.5, 3.25, 11.0])
    ref = _ref(oracle_mod, w)
    assert ref.sum() > 0
    got, st = _run(gpu_engine, w, "cellw")
    assert st["kernel_used"] == 5
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("plan", ["2,4,2,2,2", "1,4,1,1,1"])
def test_cellw_many_rechecks(gpu_engine, oracle_mod, plan, monkeypatch):
    """Copies of every atom on bin thresholds: thousands of FP64 rechecks per
    item, far more than a warp's queue holds between drains."""
    monkeypatch.setenv("ANALISI_GB300_CELLW_PLAN", plan)
    copies = 12
    w = copies_on_thresholds(copies)
    N = w["positions"].shape[1]
    ref = _ref(oracle_mod, w)
    got, st = _run(gpu_engine, w, "cellw")
    assert st["kernel_used"] == 5
    assert st["rechecks"] >= N * (copies - 1)
    np.testing.assert_array_equal(got, ref)


def test_cellw_small_boxes(gpu_engine, oracle_mod):
    """L = 10 with rmax = 4 has a grid only at reach 3 (7 cells of 1.43): the
    warp kernel takes it and counts exactly; L = 7 (L/2 < rmax) has none, and
    the forced kernel refuses."""
    from analisi_gb300 import engine
    w = workloads.small_case(64, 200, 6, 10.0, 0.1, [200], rmin=0.0, rmax=4.0, nbin=10, tmax=2,
                             skip=1, every=1, ntimesteps=3, primo=0)
    got, st = _run(gpu_engine, w, "cellw")
    assert st["kernel_used"] == 5
    np.testing.assert_array_equal(got, _ref(oracle_mod, w))
    w = workloads.small_case(64, 100, 6, 7.0, 0.1, [100], rmin=0.0, rmax=4.0, nbin=10, tmax=2,
                             skip=1, every=1, ntimesteps=3, primo=0)
    with pytest.raises(engine.GofrError):
        _run(gpu_engine, w, "cellw")


def test_cellw_windows_and_debug_free_stats(gpu_engine, oracle_mod):
    """Several calculate(primo) windows of one trajectory through the warp
    kernel (one launch per window) equal the oracle's windows."""
    seed, N, T, L, sigma, counts, params = CASES[0]
    w = workloads.small_case(seed, N, T, L, sigma, counts, **params)
    p = w["params"]
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    primos = [0, 1, 3]
    got = gpu_engine.run_windows(p["rmin"], p["rmax"], p["nbin"], 2, 2, 1, 4, primos,
                                 kernel="cellw")
    for k, pr in enumerate(primos):
        ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                      p["rmin"], p["rmax"], p["nbin"], 2, 4, 2, 1, 4, pr)
        np.testing.assert_array_equal(got[k], ref)


def _child(kernel, env):
    import json
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    out = subprocess.run([sys.executable, os.path.join(here, "tune_child.py"), kernel],
                         env={**os.environ, **env}, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    return json.loads(out.stdout.strip().splitlines()[-1])


def _want(oracle_mod):
    from tune_child import case
    w = case()
    p = w["params"]
    c = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                p["rmin"], p["rmax"], p["nbin"], p["tmax"], 8, p["skip"],
                                p["every"], p["ntimesteps"], p["primo"])
    return {"sum": int(c.sum()),
            "weighted": int((c.astype(object) * (1 + np.arange(c.size).reshape(c.shape))).sum())}


def test_tuned_choice_is_persisted_and_reused_by_auto(built_engine, oracle_mod, tmp_path):
    """GOFR_KERNEL_TUNED times the all-pairs kernel and both cell-list forms
    (the warp-streamed one with CTAs of 8 and 16 warps and one or two
    histogram copies), writes its choice to ANALISI_GB300_TUNE_CACHE; a new
    process running AUTO on the same key takes that choice without timing
    anything.  Counts are the oracle's every time."""
    want = _want(oracle_mod)
    cache, log1, log2 = (str(tmp_path / n) for n in ("cache.txt", "log1.txt", "log2.txt"))
    a = _child("tuned", {"ANALISI_GB300_TUNE_CACHE": cache, "ANALISI_GB300_TUNE_LOG": log1})
    assert {k: a[k] for k in want} == want
    timed = open(log1).read()
    assert "all-pairs" in timed and "block-cells" in timed
    assert "cta_warps=16 hcopy=2" in timed and "cta_warps=8 hcopy=1" in timed
    lines = open(cache).read().split("\n")
    key, kind = lines[0].split()[0], int(lines[0].split()[1])
    assert len(lines[0].split()) == 9
    b = _child("auto", {"ANALISI_GB300_TUNE_CACHE": cache, "ANALISI_GB300_TUNE_LOG": log2})
    assert {k: b[k] for k in want} == want
    assert b["kernel_used"] == {0: 1, 1: 3, 2: 5}[kind]
    import os
    assert not os.path.exists(log2) or open(log2).read() == ""  # nothing timed again
    assert open(cache).read().count("\n") == 1                   # nothing stored again


@pytest.mark.parametrize("shape", ["8 1", "8 2", "16 1", "16 2"])
def test_every_cta_size_and_histogram_depth_is_exact(built_engine, oracle_mod, tmp_path, shape):
    """A cache line pins the warp-streamed kernel's CTA size and histogram
    copies (through AUTO's use of the cache); each variant counts exactly."""
    want = _want(oracle_mod)
    cache = str(tmp_path / "cache.txt")
    first = _child("tuned", {"ANALISI_GB300_TUNE_CACHE": cache})
    key = open(cache).read().split()[0]
    # the warp-streamed planner's first choice for this job, with this shape
    from analisi_gb300 import engine  # noqa: F401
    with open(cache, "w") as f:
        f.write(f"{key} 2 2 4 1 1 2 {shape}\n")
    b = _child("auto", {"ANALISI_GB300_TUNE_CACHE": cache})
    assert first["sum"] == want["sum"]
    assert b["kernel_used"] == 5
    assert {k: b[k] for k in want} == want


def test_cellw_many_types(gpu_engine, oracle_mod):
    """66 types (4422 channels, one bin): the neighbour's type travels in the
    record's top byte, so the warp-streamed kernel takes any type count whose
    histogram and channel table fit shared memory; counts are the oracle's."""
    counts = [40] * 65 + [3000 - 40 * 65]
    w = workloads.small_case(66, 3000, 5, 31.0, 0.2, counts, rmin=0.5, rmax=5.0, nbin=1,
                             tmax=2, skip=1, every=1, ntimesteps=3, primo=0)
    assert w["ntypes"] == 66
    got, st = _run(gpu_engine, w, "cellw")
    assert st["kernel_used"] == 5
    np.testing.assert_array_equal(got, _ref(oracle_mod, w))
