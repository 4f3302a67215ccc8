"""The GOFR_DEBUG_BOUNDS build of the engine (device-side index checks on the
histogram, slot and range-table accesses that set an error word instead of
trapping): every kernel family runs parity cases through it with no check
firing and the oracle's counts.  The variant is compiled here into
analisi_gb300/_build_debug/ (a minute on the GPU host)."""
import numpy as np
import pytest

from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def debug_lib(built_engine):
    from analisi_gb300 import build, engine
    path = build.build_engine(debug_bounds=True)
    return engine.load_library(path)


def _ref(oracle_mod, w, p):
    return oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                   p["rmin"], p["rmax"], p["nbin"], p["tmax"], 1, p["skip"],
                                   p["every"], p["ntimesteps"], p["primo"], tric=w["triclinic"])


@pytest.mark.parametrize("kernel,tric,L,rmax", [("f32", False, 18.0, 5.0), ("f32", True, 14.0, 5.0),
                                                 ("f32", False, 6.0, 4.5),  # wrap check
                                                 ("f64", True, 14.0, 5.0), ("cell", False, 26.0, 5.0),
                                                 ("cellw", False, 26.0, 5.0),
                                                 ("cellw", True, 26.0, 5.0)])
def test_debug_build_parity_without_check_failures(debug_lib, oracle_mod, kernel, tric, L, rmax):
    from analisi_gb300 import engine
    w = workloads.small_case(95, 1500 if L > 10 else 120, 8, L, 0.2, [900, 600] if L > 10 else [70, 50],
                             tric=tric, wrap_into_cell=tric, rmin=0.0, rmax=rmax, nbin=45, tmax=3,
                             skip=2, every=1, ntimesteps=4, primo=1)
    p = w["params"]
    with engine.Engine(0, library=debug_lib) as e:
        e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        got = e.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                    p["ntimesteps"], p["primo"], kernel=kernel)
    np.testing.assert_array_equal(got, _ref(oracle_mod, w, p))


def test_debug_build_batch(debug_lib, oracle_mod):
    from analisi_gb300 import engine
    mem = [workloads.small_case(96 + k, N, 7, L, 0.2, c, rmin=0.0, rmax=4.5, nbin=40, tmax=2,
                                skip=2, every=1, ntimesteps=4, primo=0)
           for k, (N, L, c) in enumerate([(3000, 31.0, [2000, 1000]), (300, 14.0, [300]),
                                          (90, 6.0, [45, 45])])]
    trajs = []
    for w in mem:
        p = w["params"]
        trajs.append(dict(positions=w["positions"], boxes=w["boxes"], type_ids=w["type_ids"],
                          ntypes=w["ntypes"],
                          params=engine.make_params(p["rmin"], p["rmax"], p["nbin"], p["tmax"],
                                                    p["skip"], p["every"], p["ntimesteps"],
                                                    p["primo"])))
    with engine.Engine(0, library=debug_lib) as e:
        e.batch_set(trajs)
        outs = e.batch_run(use_graph=True)
    for w, got in zip(mem, outs):
        np.testing.assert_array_equal(got, _ref(oracle_mod, w, w["params"]))


@pytest.mark.parametrize("kernel", ["cell", "f32"])
def test_debug_build_recheck_queue_overflow(debug_lib, oracle_mod, kernel, monkeypatch):
    """Copies of every atom on bin thresholds: the recheck queue is drained
    between tiles and overflows into the flush's own FP64 path, with every index
    check passing."""
    from analisi_gb300 import engine
    from test_gpu_cells import copies_on_thresholds
    monkeypatch.setenv("ANALISI_GB300_CELL_PLAN", "2,3,3,3,3")
    w = copies_on_thresholds()
    p = w["params"]
    with engine.Engine(0, library=debug_lib) as e:
        e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        got = e.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                    p["ntimesteps"], p["primo"], kernel=kernel)
    np.testing.assert_array_equal(got, _ref(oracle_mod, w, p))


def test_bounded_wait_that_runs_out_reports_and_keeps_the_context(debug_lib, oracle_mod,
                                                                   monkeypatch):
    """ANALISI_GB300_DEBUG_STALL=1 (debug build only) arms the all-pairs
    kernel's first tile barrier for bytes that no copy brings: no copy is ever
    issued, so nothing is in flight when the short bounded wait gives up.  The
    run returns GOFR_ERR_DEVICE naming the bounded wait, and the same context
    then gives the oracle's counts."""
    from analisi_gb300 import engine
    w = workloads.small_case(97, 1500, 6, 18.0, 0.2, [900, 600], rmin=0.0, rmax=5.0, nbin=45,
                             tmax=2, skip=2, every=1, ntimesteps=3, primo=0)
    p = w["params"]
    args = (p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"], p["ntimesteps"],
            p["primo"])
    with engine.Engine(0, library=debug_lib) as e:
        e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        monkeypatch.setenv("ANALISI_GB300_DEBUG_STALL", "1")
        with pytest.raises(engine.GofrError) as err:
            e.run(*args, kernel="f32")
        assert err.value.code == -6 and "bounded wait ran out" in str(err.value)
        monkeypatch.delenv("ANALISI_GB300_DEBUG_STALL")
        got = e.run(*args, kernel="f32")
    np.testing.assert_array_equal(got, _ref(oracle_mod, w, p))
