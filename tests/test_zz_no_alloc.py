"""The allocation-free entry point gofr_run_f64_noalloc.

It exists for callers that cannot call cudaMalloc -- code whose device memory
is owned by a framework pool, or that must not allocate inside its loop --
and that already hold frames, types and the result buffer on the device.  It
must give exactly the counts of the regular entry point (gofr_run) and of
the oracle, on consecutive calls that share its one static scratch array, and
report a type id outside 0..ntypes-1 instead of indexing with it.

The device buffers of this test are made by torch (the test may allocate; the
entry point under test must not).  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # seed, N, T, L, sigma, counts, tric, wrap_into_cell, params
    (41, 300, 16, 12.0, 0.2, [150, 100, 50], False, False,
     dict(rmin=0.0, rmax=5.5, nbin=64, tmax=5, skip=3, every=1, ntimesteps=10, primo=1)),
    (42, 256, 12, 14.0, 0.2, [128, 128], True, True,
     dict(rmin=0.4, rmax=6.0, nbin=50, tmax=4, skip=2, every=2, ntimesteps=8, primo=0)),
]


@pytest.mark.parametrize("case", CASES, ids=["ortho", "triclinic"])
def test_noalloc_matches_gofr_run_and_oracle_twice(built_engine, oracle_mod, case):
    torch = pytest.importorskip("torch")
    from analisi_gb300 import engine, workloads
    seed, N, T, L, sigma, counts, tric, wrap, params = case
    w = workloads.small_case(seed, N, T, L, sigma, counts, tric=tric, wrap_into_cell=wrap,
                             **params)
    p = w["params"]
    with engine.Engine(0) as eng:
        eng.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                       triclinic=w["triclinic"])
        expected = eng.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                           p["ntimesteps"], p["primo"])
    assert expected.sum() > 0
    ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                  p["rmin"], p["rmax"], p["nbin"], p["tmax"], 1, p["skip"],
                                  p["every"], p["ntimesteps"], p["primo"], tric=tric)
    np.testing.assert_array_equal(expected, ref)

    torch.cuda.set_device(0)
    dpos = torch.from_numpy(np.ascontiguousarray(w["positions"])).to("cuda:0")
    dbox = torch.from_numpy(np.ascontiguousarray(w["boxes"])).to("cuda:0")
    dtyp = torch.from_numpy(np.ascontiguousarray(w["type_ids"], dtype=np.int32)).to("cuda:0")
    dout = torch.full((expected.size,), -1, dtype=torch.int64, device="cuda:0")
    torch.cuda.synchronize()

    lib = built_engine
    prm = engine.make_params(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                             p["ntimesteps"], p["primo"])
    err = ctypes.create_string_buffer(512)
    for call in range(2):
        rc = lib.gofr_run_f64_noalloc(
            ctypes.c_void_p(dpos.data_ptr()), ctypes.c_void_p(dbox.data_ptr()),
            engine.BOX_TRICLINIC if tric else engine.BOX_ORTHO, ctypes.c_void_p(dtyp.data_ptr()),
            w["ntypes"], N, T, ctypes.byref(prm), ctypes.c_void_p(dout.data_ptr()), None, err,
            len(err))
        assert rc == 0, err.value.decode()
        got = dout.cpu().numpy().view(np.uint64).reshape(expected.shape)
        np.testing.assert_array_equal(got, expected, err_msg=f"call {call}")


def test_noalloc_rejects_too_many_types(built_engine):
    torch = pytest.importorskip("torch")
    from analisi_gb300 import engine
    torch.cuda.set_device(0)
    buf = torch.zeros(64, dtype=torch.float64, device="cuda:0")
    prm = engine.make_params(0.0, 2.0, 10, 1, 1, 1, 1, 0)
    err = ctypes.create_string_buffer(512)
    ptr = ctypes.c_void_p(buf.data_ptr())
    rc = built_engine.gofr_run_f64_noalloc(ptr, ptr, engine.BOX_ORTHO, ptr, 17, 4, 2,
                                           ctypes.byref(prm), ptr, None, err, len(err))
    assert rc == -1
    assert b"1..16 types" in err.value


@pytest.mark.parametrize("bad", [2, -1, 1000])
def test_noalloc_reports_type_ids_out_of_range(built_engine, bad):
    """A caller's type id outside 0..ntypes-1 (the host never sees the ids)
    is found by the kernel: GOFR_ERR_DEVICE with a type-id message, the pairs
    of that atom skipped, and the next call with valid ids is exact again."""
    torch = pytest.importorskip("torch")
    from analisi_gb300 import engine, workloads
    w = workloads.small_case(43, 200, 8, 11.0, 0.2, [100, 100], rmin=0.0, rmax=5.0, nbin=40,
                             tmax=2, skip=2, every=1, ntimesteps=4, primo=0)
    p = w["params"]
    with engine.Engine(0) as eng:
        eng.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        expected = eng.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                           p["ntimesteps"], p["primo"])
    torch.cuda.set_device(0)
    dpos = torch.from_numpy(np.ascontiguousarray(w["positions"])).to("cuda:0")
    dbox = torch.from_numpy(np.ascontiguousarray(w["boxes"])).to("cuda:0")
    good = np.ascontiguousarray(w["type_ids"], dtype=np.int32)
    bad_ids = good.copy()
    bad_ids[57] = bad
    dout = torch.zeros((expected.size,), dtype=torch.int64, device="cuda:0")
    prm = engine.make_params(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                             p["ntimesteps"], p["primo"])
    err = ctypes.create_string_buffer(512)

    def call(ids):
        dtyp = torch.from_numpy(ids).to("cuda:0")
        torch.cuda.synchronize()
        return built_engine.gofr_run_f64_noalloc(
            ctypes.c_void_p(dpos.data_ptr()), ctypes.c_void_p(dbox.data_ptr()), engine.BOX_ORTHO,
            ctypes.c_void_p(dtyp.data_ptr()), w["ntypes"], 200, 8, ctypes.byref(prm),
            ctypes.c_void_p(dout.data_ptr()), None, err, len(err))

    assert call(bad_ids) == -6
    assert b"type id" in err.value
    assert call(good) == 0, err.value.decode()
    got = dout.cpu().numpy().view(np.uint64).reshape(expected.shape)
    np.testing.assert_array_equal(got, expected)
