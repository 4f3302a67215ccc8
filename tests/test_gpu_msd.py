"""Mean square displacement on the GPU (gofr_msd_run, the drop-in
pyanalisi.MeanSquareDisplacement) against the reference's own results
(tests/golden/msd) and the oracle's restatement of MSD::calc_single_th.

The reference keeps a running mean per (lag, type); the GPU forms every
squared displacement with the reference's FP64 operations, sums them in a
fixed order and divides by the count.  The two agree to rounding: the tests
use a relative tolerance of 1e-12 (the running mean's own error for these
term counts is ~1e-15 to 1e-13)."""
import numpy as np
import pytest

import golden_util as gu
from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def pa(built_engine):
    from analisi_gb300 import build
    build.build_host()
    import analisi_gb300
    return analisi_gb300.load_pyanalisi()


@pytest.mark.parametrize("name", gu.msd_names())
def test_engine_msd_matches_reference(gpu_engine, name):
    d = gu.load_msd(name)
    m = d["meta"]
    box = np.zeros((d["internal_positions"].shape[0], 6))
    box[:, 3:6] = 50.0
    gpu_engine.set_frames(d["internal_positions"], box, d["internal_type_ids"], m["ntypes"])
    gpu_engine.set_centres(d["internal_centres"])
    out = gpu_engine.msd(m["skip"], m["tmax"], m["ntimesteps"], m["primo"], m["cm_msd"],
                         m["cm_self"])
    np.testing.assert_allclose(out, d["ref_buffer"], rtol=RTOL, atol=0)


@pytest.mark.parametrize("name", gu.msd_names())
def test_pyanalisi_msd_matches_reference(pa, name):
    """The drop-in class on the caller's raw arrays, as the reference's
    tests/test_msd.py calls it."""
    d = gu.load_msd(name)
    m = d["meta"]
    t = pa.Trajectory(d["positions"], np.zeros_like(d["positions"]), d["types"], d["box"],
                      getattr(pa.BoxFormat, m["box_format"]), m["wrap"], False)
    with pa.MeanSquareDisplacement(t, m["skip"], m["tmax"], m["nthreads"], m["cm_msd"],
                                   m["cm_self"], False) as msd:
        msd.reset(m["ntimesteps"])
        msd.calculate(m["primo"])
        out = np.array(msd, copy=True)
    assert out.shape == d["ref_buffer"].shape
    np.testing.assert_allclose(out, d["ref_buffer"], rtol=RTOL, atol=0)


@pytest.mark.parametrize("cm_msd,cm_self", [(False, False), (True, False), (False, True),
                                            (True, True)])
def test_engine_msd_matches_oracle_larger(gpu_engine, oracle_mod, cm_msd, cm_self):
    """3000 atoms in 3 types (uneven, interleaved), 120 frames, 40 lags, skip 3."""
    w = workloads.small_case(71, 3000, 120, 30.0, 0.2, [1700, 900, 400])
    rng = np.random.default_rng(72)
    tids = rng.permutation(w["type_ids"]).astype(np.int32)
    pos = w["positions"]
    cm = oracle_mod.centres(pos, tids, 3)
    ref = oracle_mod.msd(pos, tids, 3, 3, 40, 70, 5, cm_msd, cm_self, cm=cm)
    gpu_engine.set_frames(pos, w["boxes"], tids, 3)
    gpu_engine.set_centres(cm)
    out = gpu_engine.msd(3, 40, 70, 5, cm_msd, cm_self)
    np.testing.assert_allclose(out, ref, rtol=RTOL, atol=0)
    st = gpu_engine.stats()
    assert st["pairs"] == 40 * 24 * 3000  # leff x origins x atoms


def test_msd_errors(gpu_engine, pa):
    from analisi_gb300 import engine
    w = workloads.small_case(73, 100, 20, 10.0, 0.1, [60, 40])
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], 2)
    with pytest.raises(engine.GofrError, match="centre"):
        gpu_engine.msd(1, 5, 10, 0, True, False)  # no centres uploaded
    with pytest.raises(engine.GofrError, match="too short"):
        gpu_engine.msd(1, 5, 16, 0)  # 5 + 16 > 20 frames
    out = gpu_engine.msd(1, 5, 15, 0)  # 5 + 15 = 20: the largest accepted
    assert out.shape == (5, 1, 2) and np.all(out[0] == 0.0)
    d = gu.load_msd(gu.msd_names()[0])
    t = pa.Trajectory(d["positions"], np.zeros_like(d["positions"]), d["types"], d["box"],
                      pa.BoxFormat.LammpsOrtho, False, False)
    msd = pa.MeanSquareDisplacement(t, 1, 10, 1, False, False, False)
    msd.reset(d["positions"].shape[0])
    with pytest.raises(RuntimeError, match="too short"):
        msd.calculate(0)
