"""Cell-list form of the FP32 kernel (GOFR_KERNEL_CELL): same exact counts as
the oracle and as the all-pairs kernels, for boxes with at least 3 cells of
edge >= rmax per axis (unwrapped coordinates, shifted and non-cubic boxes,
several types, skip/every/primo)."""
import numpy as np
import pytest

from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu

CASES = [
    # seed, N, T, L, sigma, counts, params
    (61, 2000, 10, 27.0, 0.3, [1200, 500, 300],
     dict(rmin=0.0, rmax=6.0, nbin=60, tmax=3, skip=3, every=1, ntimesteps=6, primo=1)),
    (62, 3000, 8, 31.0, 0.2, [3000],
     dict(rmin=0.5, rmax=5.1, nbin=37, tmax=2, skip=2, every=1, ntimesteps=5, primo=0)),
    (63, 2500, 9, 29.5, 0.25, [1000, 1000, 500],
     dict(rmin=0.0, rmax=4.0, nbin=80, tmax=4, skip=4, every=2, ntimesteps=5, primo=0)),
]


def _run(eng, w, kernel):
    p = w["params"]
    eng.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
    c = eng.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                p["ntimesteps"], p["primo"], kernel=kernel)
    return c, eng.stats()


# Cell-list configurations "reach,r,bx,by,bz" forced through
# ANALISI_GB300_CELL_PLAN (None = the planner's choice): cells of edge
# >= rmax (reach 1) and >= rmax/2 (reach 2), 2/3/4 first atoms per thread,
# single cells and blocks whose neighbourhood wraps the box.
PLANS = [None, "1,4,1,1,1", "1,2,2,1,1", "2,2,1,1,1", "2,3,2,1,3", "2,4,3,3,3"]


@pytest.mark.parametrize("plan", PLANS, ids=[str(p) for p in PLANS])
@pytest.mark.parametrize("case", CASES, ids=[str(c[0]) for c in CASES])
def test_cells_match_oracle_and_all_pairs(gpu_engine, oracle_mod, case, plan, monkeypatch):
    if plan is None:
        monkeypatch.delenv("ANALISI_GB300_CELL_PLAN", raising=False)
    else:
        monkeypatch.setenv("ANALISI_GB300_CELL_PLAN", plan)
    seed, N, T, L, sigma, counts, params = case
    w = workloads.small_case(seed, N, T, L, sigma, counts, **params)
    if seed == 62:  # shifted, non-cubic box
        w["boxes"] = w["boxes"].copy()
        w["boxes"][:, 0] -= 3.0
        w["boxes"][:, 4] *= 1.08
    p = w["params"]
    ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                  p["rmin"], p["rmax"], p["nbin"], p["tmax"], 8, p["skip"],
                                  p["every"], p["ntimesteps"], p["primo"])
    cell, st = _run(gpu_engine, w, "cell")
    assert st["kernel_used"] == 3
    # the planner may take the whole box as one block for so few atoms
    assert st["evaluated"] <= st["pairs"] if plan is None else st["evaluated"] < st["pairs"]
    np.testing.assert_array_equal(cell, ref)
    allp, _ = _run(gpu_engine, w, "f32")
    np.testing.assert_array_equal(allp, ref)


@pytest.mark.parametrize("plan", [None, "1,3,1,1,1", "2,2,1,2,1", "2,4,2,2,2"],
                         ids=["auto", "1,3,1,1,1", "2,2,1,2,1", "2,4,2,2,2"])
def test_cells_far_unwrapped_coordinates(gpu_engine, oracle_mod, plan, monkeypatch):
    """Atoms several box lengths outside the cell (the reference iterates its
    minimum image), a box not at the origin and the all-wrapped neighbour
    images: the cell path wraps every coordinate into the box first and must
    still count exactly what the oracle counts."""
    if plan is None:
        monkeypatch.delenv("ANALISI_GB300_CELL_PLAN", raising=False)
    else:
        monkeypatch.setenv("ANALISI_GB300_CELL_PLAN", plan)
    w = workloads.small_case(65, 2400, 7, 26.0, 0.4, [1500, 900], rmin=0.3, rmax=5.0, nbin=45,
                             tmax=3, skip=2, every=1, ntimesteps=4, primo=0)
    rng = np.random.default_rng(650)
    L = 26.0
    w["positions"] = w["positions"] + L * rng.integers(-4, 5, size=(1, 2400, 3))
    w["boxes"] = w["boxes"].copy()
    w["boxes"][:, 0:3] += np.array([-7.5, 3.25, 11.0])
    w["positions"] = w["positions"] + np.array([-7.5, 3.25, 11.0])
    p = w["params"]
    ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                  p["rmin"], p["rmax"], p["nbin"], p["tmax"], 8, p["skip"],
                                  p["every"], p["ntimesteps"], p["primo"])
    assert ref.sum() > 0
    cell, st = _run(gpu_engine, w, "cell")
    assert st["kernel_used"] == 3
    np.testing.assert_array_equal(cell, ref)


def test_cell_kernel_refuses_small_box(gpu_engine):
    from analisi_gb300 import engine
    w = workloads.small_case(64, 200, 6, 10.0, 0.1, [200], rmin=0.0, rmax=4.0, nbin=10, tmax=2,
                             skip=1, every=1, ntimesteps=3, primo=0)
    with pytest.raises(engine.GofrError):
        _run(gpu_engine, w, "cell")


def test_tuned_kernel_choice_is_exact_and_cached(gpu_engine, oracle_mod, tmp_path, monkeypatch):
    """GOFR_KERNEL_TUNED times the all-pairs and cell-list forms on a sample and
    keeps the fastest; whichever wins, the counts are the oracle's, and the
    choice is written to the cache file named by ANALISI_GB300_TUNE_CACHE."""
    seed, N, T, L, sigma, counts, params = CASES[0]
    w = workloads.small_case(seed, N, T, L, sigma, counts, **params)
    p = w["params"]
    ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                  p["rmin"], p["rmax"], p["nbin"], p["tmax"], 8, p["skip"],
                                  p["every"], p["ntimesteps"], p["primo"])
    a, st = _run(gpu_engine, w, "tuned")
    np.testing.assert_array_equal(a, ref)
    assert st["kernel_used"] in (1, 3, 5)
    b, st2 = _run(gpu_engine, w, "tuned")
    np.testing.assert_array_equal(b, ref)
    assert st2["kernel_used"] == st["kernel_used"]


def copies_on_thresholds(copies=12, distinct=600):
    """A 2-type random walk whose atoms each have `copies` copies spaced by 0.5
    along x (the same trajectory shifted), with rmin = dr = 0.5: at lag 0 every
    pair of copies lies on a bin threshold, where the reference's bin depends on
    the last bit of its FP64 arithmetic and FP32 cannot certify anything."""
    w = workloads.small_case(66, distinct, 6, 30.0, 0.3, [distinct // 2, distinct - distinct // 2],
                             rmin=0.5, rmax=6.0, nbin=11, tmax=3, skip=1, every=1,
                             ntimesteps=4, primo=0)
    pos = np.repeat(w["positions"], copies, axis=1)
    pos[..., 0] += np.tile(0.5 * np.arange(copies), distinct)
    w["positions"] = np.ascontiguousarray(pos)
    w["type_ids"] = np.ascontiguousarray(np.repeat(w["type_ids"], copies))
    return w


@pytest.mark.parametrize("kernel,plan", [("cell", "2,3,3,3,3"), ("cell", "1,4,1,1,1"),
                                         ("f32", None)],
                         ids=["cell-2,3,3,3,3", "cell-1,4,1,1,1", "all-pairs"])
def test_many_rechecks_drain_the_queue(gpu_engine, oracle_mod, kernel, plan, monkeypatch):
    """Thousands of FP64 rechecks per lag-0 work item, more than a CTA's recheck
    queue holds within one tile: the queue is drained between tiles and the
    flush recomputes what does not fit; the counts must still be the oracle's."""
    if plan is None:
        monkeypatch.delenv("ANALISI_GB300_CELL_PLAN", raising=False)
    else:
        monkeypatch.setenv("ANALISI_GB300_CELL_PLAN", plan)
    copies = 12
    w = copies_on_thresholds(copies)
    N = w["positions"].shape[1]
    p = w["params"]
    ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                  p["rmin"], p["rmax"], p["nbin"], p["tmax"], 8, p["skip"],
                                  p["every"], p["ntimesteps"], p["primo"])
    got, st = _run(gpu_engine, w, kernel)
    assert st["kernel_used"] == (3 if kernel == "cell" else 1)
    # at lag 0 every ordered pair of copies sits on a threshold and is rechecked
    assert st["rechecks"] >= N * (copies - 1)
    np.testing.assert_array_equal(got, ref)
