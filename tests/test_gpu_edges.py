"""Edge cases against the oracle (the C restatement of the reference): ragged
and degenerate sizes, parameters at their limits, values on decision
boundaries, and inputs the reference cannot handle (rejected up front)."""
import numpy as np
import pytest

from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu


def _check(eng, oracle_mod, pos, boxes, tids, ntypes, kernels=("auto", "f64"), **p):
    tric = boxes.shape[1] == 9
    ref = oracle_mod.gofrt_counts(pos, boxes, tids, ntypes, p["rmin"], p["rmax"], p["nbin"],
                                  p["tmax"], 1, p["skip"], p["every"], p["ntimesteps"], p["primo"],
                                  tric=tric)
    eng.set_frames(pos, boxes, tids, ntypes, triclinic=tric)
    for k in kernels:
        got = eng.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                      p["ntimesteps"], p["primo"], kernel=k)
        np.testing.assert_array_equal(got, ref, err_msg=k)
    return ref


def _walk(seed, N, T, L, sigma=0.2, ntypes=2, tric=False):
    w = workloads.small_case(seed, N, T, L, sigma, [N // ntypes + N % ntypes] +
                             [N // ntypes] * (ntypes - 1), tric=tric)
    return w["positions"], w["boxes"], w["type_ids"], w["ntypes"]


@pytest.mark.parametrize("p", [
    dict(rmin=0.0, rmax=2.0, nbin=10, tmax=1, skip=1, every=1, ntimesteps=1, primo=0),    # one frame
    dict(rmin=0.0, rmax=2.0, nbin=1, tmax=3, skip=1, every=1, ntimesteps=5, primo=0),     # one bin
    dict(rmin=0.0, rmax=3.0, nbin=20, tmax=3, skip=9, every=1, ntimesteps=5, primo=0),    # skip > n
    dict(rmin=0.0, rmax=3.0, nbin=20, tmax=4, skip=1, every=7, ntimesteps=6, primo=0),    # every > leff
    dict(rmin=0.0, rmax=3.0, nbin=20, tmax=50, skip=2, every=1, ntimesteps=6, primo=0),   # tmax > n
    dict(rmin=0.0, rmax=3.0, nbin=20, tmax=0, skip=3, every=2, ntimesteps=7, primo=2),    # tmax = 0
    dict(rmin=0.0, rmax=3.0, nbin=20, tmax=4, skip=1, every=1, ntimesteps=12, primo=0),   # leff+n+primo = T+1
    dict(rmin=2.5, rmax=1.0, nbin=20, tmax=2, skip=1, every=1, ntimesteps=4, primo=0),    # rmin > rmax
    dict(rmin=-1.0, rmax=2.5, nbin=35, tmax=2, skip=1, every=1, ntimesteps=4, primo=0),   # rmin < 0
    dict(rmin=0.0, rmax=3.0, nbin=1 << 24, tmax=1, skip=1, every=1, ntimesteps=1, primo=0),  # huge nbin
])
def test_parameter_limits(gpu_engine, oracle_mod, p):
    pos, boxes, tids, nt = _walk(3, 40, 16, 6.0)
    if p["nbin"] > 1_000_000:
        # a huge histogram: only one lag and a single type so the output stays small
        pos, boxes, tids, nt = _walk(3, 20, 4, 6.0, ntypes=1)
        _check(gpu_engine, oracle_mod, pos, boxes, tids, nt, kernels=("auto",), **p)
        st = gpu_engine.stats()
        assert st["kernel_used"] == 2   # bin map beyond FP32 certification: FP64 kernel
        return
    _check(gpu_engine, oracle_mod, pos, boxes, tids, nt, **p)


@pytest.mark.parametrize("N", [1, 2, 3, 17, 1023, 1025])
def test_ragged_atom_counts(gpu_engine, oracle_mod, N):
    pos, boxes, tids, nt = _walk(N, N, 8, 9.0, ntypes=min(2, N))
    _check(gpu_engine, oracle_mod, pos, boxes, tids, nt,
           rmin=0.0, rmax=4.0, nbin=25, tmax=3, skip=2, every=1, ntimesteps=5, primo=0)


def test_distances_on_bin_edges_and_half_box(gpu_engine, oracle_mod):
    """Pairs placed exactly at bin-edge distances, at rmax, at l/2 (not wrapped,
    strict '>'), and just above l/2 (wrapped)."""
    L = 8.0
    ds = [0.0, 0.1, 0.2, 0.3, 0.5, 1.0, 2.0, 2.9999999999, 3.0, 4.0, 4.000000001, 3.9999999]
    T = len(ds)
    pos = np.zeros((T, 4, 3))
    for f, d in enumerate(ds):
        pos[f, 0] = [1.0, 2.0, 3.0]
        pos[f, 1] = [1.0 + d, 2.0, 3.0]
        pos[f, 2] = [1.0, 2.0 + d, 3.0 - d]
        pos[f, 3] = [1.0 - d, 2.0 - d / 2, 3.0 + d / 3]
    boxes = workloads.lammps_to_internal(np.tile([0, L, 0, L, 0, L], (T, 1)).astype(float))
    tids = np.array([0, 1, 0, 1], dtype=np.int32)
    for rmax, nbin in [(3.0, 30), (4.0, 40), (5.0, 7)]:
        _check(gpu_engine, oracle_mod, pos, boxes, tids, 2, rmin=0.0, rmax=rmax, nbin=nbin,
               tmax=3, skip=1, every=1, ntimesteps=T - 2, primo=0)


def test_atoms_many_boxes_away(gpu_engine, oracle_mod):
    """Unwrapped coordinates several box lengths outside the cell (multi-step
    minimum image), orthorhombic and triclinic."""
    for tric in (False, True):
        pos, boxes, tids, nt = _walk(9, 60, 10, 7.0, tric=tric)
        shift = np.random.default_rng(1).integers(-4, 5, (1, 60, 3)) * 7.0
        _check(gpu_engine, oracle_mod, pos + shift, boxes, tids, nt,
               rmin=0.0, rmax=3.2, nbin=32, tmax=3, skip=2, every=1, ntimesteps=6, primo=1)


def test_nonfinite_coordinates_rejected(gpu_engine):
    from analisi_gb300 import engine
    pos, boxes, tids, nt = _walk(4, 10, 3, 5.0)
    pos = pos.copy()
    pos[1, 3, 2] = np.nan
    with pytest.raises(engine.GofrError, match="non-finite"):
        gpu_engine.set_frames(pos, boxes, tids, nt)
    pos[1, 3, 2] = np.inf
    with pytest.raises(engine.GofrError, match="non-finite"):
        gpu_engine.set_frames(pos, boxes, tids, nt)


def test_bad_boxes_and_types_rejected(gpu_engine):
    from analisi_gb300 import engine
    pos, boxes, tids, nt = _walk(5, 10, 3, 5.0)
    b = boxes.copy()
    b[0, 4] = 0.0
    with pytest.raises(engine.GofrError, match="not positive"):
        gpu_engine.set_frames(pos, b, tids, nt)
    t = tids.copy()
    t[0] = 7
    with pytest.raises(engine.GofrError, match="type id"):
        gpu_engine.set_frames(pos, boxes, t, nt)
