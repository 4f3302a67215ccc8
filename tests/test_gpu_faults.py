"""Failure paths of the C ABI, injected on the host (no GPU fault): device
allocations made to fail through the ANALISI_GB300_FAIL_ALLOC hook return
GOFR_ERR_NOMEM with a message, leak nothing the context keeps, and leave the
context usable: the next call without the hook gives the oracle's counts."""
import numpy as np
import pytest

from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu


def _case():
    return workloads.small_case(91, 600, 8, 16.0, 0.2, [400, 200], rmin=0.0, rmax=5.0, nbin=50,
                                tmax=3, skip=2, every=1, ntimesteps=4, primo=0)


def test_context_creation_failure_is_clean(built_engine, monkeypatch):
    from analisi_gb300 import engine
    monkeypatch.setenv("ANALISI_GB300_FAIL_ALLOC", "1")
    with pytest.raises(engine.GofrError):
        engine.Engine(0)
    monkeypatch.delenv("ANALISI_GB300_FAIL_ALLOC")
    with engine.Engine(0):
        pass


def test_upload_and_run_failures_leave_context_usable(built_engine, oracle_mod, monkeypatch):
    from analisi_gb300 import engine
    w = _case()
    p = w["params"]
    ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                  p["rmin"], p["rmax"], p["nbin"], p["tmax"], 1, p["skip"],
                                  p["every"], p["ntimesteps"], p["primo"])
    with engine.Engine(0) as e:
        monkeypatch.setenv("ANALISI_GB300_FAIL_ALLOC", "1")
        with pytest.raises(engine.GofrError) as err:
            e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        assert err.value.code == -4 and "memory" in str(err.value)
        with pytest.raises(engine.GofrError):  # nothing uploaded: a state error
            e.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], 1, p["ntimesteps"], 0)
        monkeypatch.delenv("ANALISI_GB300_FAIL_ALLOC")
        e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        # the counts buffer is allocated at the first run: make that one fail
        monkeypatch.setenv("ANALISI_GB300_FAIL_ALLOC", "1")
        with pytest.raises(engine.GofrError) as err:
            e.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], 1, p["ntimesteps"], 0)
        assert err.value.code == -4
        monkeypatch.delenv("ANALISI_GB300_FAIL_ALLOC")
        got = e.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], 1, p["ntimesteps"], 0)
        np.testing.assert_array_equal(got, ref)


def test_msd_and_neighbour_allocation_failures(built_engine, oracle_mod, monkeypatch):
    from analisi_gb300 import engine
    w = _case()
    with engine.Engine(0) as e:
        e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        monkeypatch.setenv("ANALISI_GB300_FAIL_ALLOC", "1")
        with pytest.raises(engine.GofrError) as err:
            e.msd(1, 3, 4, 0)
        assert err.value.code == -4
        with pytest.raises(engine.GofrError) as err:
            e.neighbours(0, [(40, 9.0, 10.0), (40, 9.0, 10.0)], True)
        assert err.value.code == -4
        monkeypatch.delenv("ANALISI_GB300_FAIL_ALLOC")
        ref = oracle_mod.msd(w["positions"], w["type_ids"], w["ntypes"], 1, 3, 4, 0)
        np.testing.assert_allclose(e.msd(1, 3, 4, 0), ref, rtol=1e-12, atol=0)
        o = oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], w["ntypes"], 0,
                                  [(40, 9.0, 10.0), (40, 9.0, 10.0)], True)
        nl = e.neighbours(0, [(40, 9.0, 10.0), (40, 9.0, 10.0)], True)
        for a in range(0, 600, 13):
            np.testing.assert_array_equal(nl.idx(a, 1), o.idx(a, 1))


def _cell_case():
    # 6000 atoms at density ~0.094 with rmax=5: the planner takes cell lists
    return workloads.small_case(92, 6000, 6, 40.0, 0.15, [3000, 2000, 1000], rmin=0.0, rmax=5.0,
                                nbin=50, tmax=2, skip=2, every=1, ntimesteps=3, primo=0)


def test_cell_lists_that_cannot_be_allocated_fall_back(built_engine, oracle_mod, monkeypatch):
    """Only the cell-list allocations fail (ANALISI_GB300_FAIL_ALLOC=cells):
    an AUTO run and the neighbour lists take the all-pairs form with the same
    results, forced cell-list runs (both forms) report the shortage, and once
    memory is back the next calls use cell lists again."""
    from analisi_gb300 import engine
    w = _cell_case()
    p = w["params"]
    ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                  p["rmin"], p["rmax"], p["nbin"], p["tmax"], 8, p["skip"],
                                  p["every"], p["ntimesteps"], p["primo"])
    spec = [(60, 3.0 ** 2, 3.5 ** 2)] * w["ntypes"]
    oref = oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], w["ntypes"], 1, spec,
                                 True)
    args = (p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"], p["ntimesteps"],
            p["primo"])
    with engine.Engine(0) as e:
        e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        monkeypatch.setenv("ANALISI_GB300_FAIL_ALLOC", "cells")
        got = e.run(*args, kernel="auto")
        assert e.stats()["kernel_used"] == 1
        np.testing.assert_array_equal(got, ref)
        for forced in ("cell", "cellw"):
            with pytest.raises(engine.GofrError) as err:
                e.run(*args, kernel=forced)
            assert err.value.code == -4
        nl = e.neighbours(1, spec, True)
        assert e.stats()["kernel_used"] == -1  # all-pairs form
        for a in range(0, 6000, 37):
            for k in range(w["ntypes"]):
                np.testing.assert_array_equal(nl.idx(a, k), oref.idx(a, k))
        monkeypatch.delenv("ANALISI_GB300_FAIL_ALLOC")
        got = e.run(*args, kernel="auto")
        assert e.stats()["kernel_used"] in (3, 5)  # a cell-list form
        np.testing.assert_array_equal(got, ref)
        nl = e.neighbours(1, spec, True)
        assert e.stats()["kernel_used"] == -2  # cell-list form
        for a in range(0, 6000, 37):
            for k in range(w["ntypes"]):
                np.testing.assert_array_equal(nl.idx(a, k), oref.idx(a, k))


def test_planner_keeps_cells_for_dense_boxes_and_all_pairs_for_sparse(built_engine,
                                                                       oracle_mod):
    """The cap of 6 cells per atom leaves dense boxes on the cell-list kernel
    and sends a sparse box (a grid of far more cells than atoms) to the
    all-pairs kernel; both give the oracle's counts."""
    from analisi_gb300 import engine
    dense = _cell_case()
    sparse = workloads.small_case(93, 60, 6, 60.0, 0.3, [40, 20], rmin=0.0, rmax=5.0, nbin=40,
                                  tmax=2, skip=2, every=1, ntimesteps=3, primo=0)
    with engine.Engine(0) as e:
        for w, want in ((dense, (3, 5)), (sparse, (1,))):
            p = w["params"]
            e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
            got = e.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                        p["ntimesteps"], p["primo"], kernel="auto")
            assert e.stats()["kernel_used"] in want
            ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"],
                                          w["ntypes"], p["rmin"], p["rmax"], p["nbin"],
                                          p["tmax"], 4, p["skip"], p["every"], p["ntimesteps"],
                                          p["primo"])
            np.testing.assert_array_equal(got, ref)
