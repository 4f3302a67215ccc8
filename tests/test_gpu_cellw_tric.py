"""Warp-streamed cell-list kernel in triclinic boxes.

The reference's minimum image in a triclinic cell (z, then y, then x;
lib/include/basetrajectory.h:224-268) leaves every component within half the
box edge, so a pair it counts has exactly one lattice image within rmax; the
kernel bins atoms reduced into the cell's axis-aligned fundamental domain and
reaches, per warp block, every cell image within rmax, layers and rows shifted
by the tilts.  Counts must equal the oracle's (the C restatement of
lib/src/gofrt.cpp:96-122 with the triclinic minimum image) for positive,
negative and half-box tilts, non-cubic and shifted boxes, atoms several
lattice vectors outside the cell, reach 1 to 3 and several warp-block shapes;
tilts too large for the kernel's image table are refused."""
import numpy as np
import pytest

from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu


def tric_case(seed, N, T, L3, tilt, sigma, counts, lo=(0.0, 0.0, 0.0), unwrap=0, **params):
    """Random walk in the cell a=(Lx,0,0), b=(xy,Ly,0), c=(xz,yz,Lz) at lo;
    unwrap > 0 moves every atom by a fixed random lattice vector with
    components in -unwrap..unwrap."""
    rng = np.random.default_rng(seed)
    types = np.repeat(np.arange(len(counts), dtype=np.int32), counts)
    rng.shuffle(types)
    Lx, Ly, Lz = L3
    xy, xz, yz = tilt
    H = np.array([[Lx, xy, xz], [0.0, Ly, yz], [0.0, 0.0, Lz]])  # columns a, b, c
    pos = np.empty((T, N, 3))
    pos[0] = rng.uniform(0.0, 1.0, size=(N, 3)) @ H.T + np.array(lo)
    steps = rng.normal(0.0, sigma, size=(T - 1, N, 3))
    pos[1:] = pos[0] + np.cumsum(steps, axis=0)
    if unwrap:
        k = rng.integers(-unwrap, unwrap + 1, size=(N, 3)).astype(np.float64)
        pos += (k @ H.T)[None]
    row = np.array([lo[0], lo[0] + Lx, lo[1], lo[1] + Ly, lo[2], lo[2] + Lz, xy, xz, yz])
    box_lammps = np.tile(row, (T, 1))
    type_ids, ntypes = workloads.dense_type_ids(types)
    return {"positions": pos, "boxes": workloads.lammps_to_internal(box_lammps),
            "type_ids": type_ids, "ntypes": ntypes, "triclinic": True, "params": params}


def _params(rmax, nbin, rmin=0.0, tmax=3, skip=2, every=1, ntimesteps=4, primo=0):
    return dict(rmin=rmin, rmax=rmax, nbin=nbin, tmax=tmax, skip=skip, every=every,
                ntimesteps=ntimesteps, primo=primo)


# (seed, N, T, (Lx, Ly, Lz), (xy, xz, yz), sigma, counts, lo, unwrap, params)
CASES = [
    (81, 3000, 7, (30.0, 30.0, 30.0), (9.0, 6.0, 3.0), 0.3, [1800, 1200], (0.0, 0.0, 0.0), 0,
     _params(7.0, 50, rmin=0.5)),
    (82, 2600, 6, (26.0, 31.0, 35.0), (-8.0, 11.0, -13.0), 0.4, [1000, 900, 700],
     (-3.0, 2.5, 7.0), 0, _params(6.0, 40)),
    (83, 2000, 6, (24.0, 24.0, 24.0), (12.0, -12.0, 12.0), 0.3, [2000], (0.0, 0.0, 0.0), 0,
     _params(5.0, 33, rmin=0.2)),
    (84, 2400, 7, (27.0, 25.0, 29.0), (5.5, -7.25, 9.5), 0.5, [1500, 900], (4.0, -6.0, 1.5), 3,
     _params(5.5, 45, rmin=0.3)),
]
# "reach,r,wx,wy,wz" through ANALISI_GB300_CELLW_PLAN (None: the planner's
# choice; a plan the planner does not list for a case falls back to its choice)
PLANS = [None, "1,4,1,1,1", "2,4,1,2,2", "2,4,2,1,1", "3,4,2,2,2", "3,4,1,1,1"]


def _ref(oracle_mod, w):
    p = w["params"]
    return oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                   p["rmin"], p["rmax"], p["nbin"], p["tmax"], 8, p["skip"],
                                   p["every"], p["ntimesteps"], p["primo"], tric=True)


def _run(eng, w, kernel):
    p = w["params"]
    eng.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"], triclinic=True)
    c = eng.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                p["ntimesteps"], p["primo"], kernel=kernel)
    return c, eng.stats()


@pytest.mark.parametrize("plan", PLANS, ids=[str(p) for p in PLANS])
@pytest.mark.parametrize("case", CASES, ids=[str(c[0]) for c in CASES])
def test_cellw_triclinic_matches_oracle(gpu_engine, oracle_mod, case, plan, monkeypatch):
    if plan is None:
        monkeypatch.delenv("ANALISI_GB300_CELLW_PLAN", raising=False)
    else:
        monkeypatch.setenv("ANALISI_GB300_CELLW_PLAN", plan)
    seed, N, T, L3, tilt, sigma, counts, lo, unwrap, params = case
    w = tric_case(seed, N, T, L3, tilt, sigma, counts, lo=lo, unwrap=unwrap, **params)
    ref = _ref(oracle_mod, w)
    assert ref.sum() > 0
    got, st = _run(gpu_engine, w, "cellw")
    assert st["kernel_used"] == 5
    assert st["evaluated"] < st["pairs"]
    np.testing.assert_array_equal(got, ref)


def test_triclinic_auto_and_all_pairs_agree(gpu_engine, oracle_mod):
    """The default plan, the all-pairs FP32 kernel and plain FP64 on a case of
    each tilt sign: identical counts, equal to the oracle's."""
    for case in CASES[:2]:
        seed, N, T, L3, tilt, sigma, counts, lo, unwrap, params = case
        w = tric_case(seed, N, T, L3, tilt, sigma, counts, lo=lo, unwrap=unwrap, **params)
        ref = _ref(oracle_mod, w)
        for k in ("auto", "f32", "f64"):
            got, st = _run(gpu_engine, w, k)
            np.testing.assert_array_equal(got, ref)


def test_triclinic_tilt_beyond_the_image_table_is_refused(gpu_engine, oracle_mod):
    """xy = 2.7 Lx reaches x images three box lengths away: the warp kernel
    refuses the box, the default plan takes the all-pairs kernel, exactly."""
    from analisi_gb300 import engine
    w = tric_case(85, 1200, 8, (20.0, 20.0, 20.0), (54.0, 0.0, 0.0), 0.3, [1200],
                  **_params(4.0, 20))
    with pytest.raises(engine.GofrError, match="cell lists"):
        _run(gpu_engine, w, "cellw")
    got, st = _run(gpu_engine, w, "auto")
    assert st["kernel_used"] in (1, 2)
    np.testing.assert_array_equal(got, _ref(oracle_mod, w))


def test_triclinic_windows(gpu_engine, oracle_mod):
    """Several calculate(primo) windows through the warp kernel in one call."""
    seed, N, T, L3, tilt, sigma, counts, lo, unwrap, params = CASES[1]
    w = tric_case(seed, N, T, L3, tilt, sigma, counts, lo=lo, unwrap=unwrap, **params)
    p = w["params"]
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"], triclinic=True)
    primos = [0, 1, 2]
    got = gpu_engine.run_windows(p["rmin"], p["rmax"], p["nbin"], 2, 2, 1, 3, primos,
                                 kernel="cellw")
    for k, pr in enumerate(primos):
        ref = oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                      p["rmin"], p["rmax"], p["nbin"], 2, 4, 2, 1, 3, pr,
                                      tric=True)
        np.testing.assert_array_equal(got[k], ref)
