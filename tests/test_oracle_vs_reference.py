"""The C restatement against the reference's own build on random seeded
inputs (runs only where oracle/_ref was built from the reference sources;
oracle/build_ref.sh)."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")
HAVE_REF = bool(glob.glob(os.path.join(REF_DIR, "pyanalisi_ref*.so")))

pytestmark = pytest.mark.skipif(not HAVE_REF, reason="reference build (oracle/_ref) not present")


@pytest.fixture(scope="module")
def ref():
    sys.path.insert(0, REF_DIR)
    import pyanalisi_ref
    return pyanalisi_ref


@pytest.mark.parametrize("seed", range(6))
def test_random_cases_bit_exact(ref, oracle_mod, seed):
    rng = np.random.default_rng(seed)
    N = int(rng.integers(8, 60))
    T = int(rng.integers(12, 30))
    L = float(rng.uniform(4, 9))
    tric = bool(seed % 2)
    wrap = bool((seed // 2) % 2) or tric   # LammpsTriclinic needs wrap=True (see golden notes)
    pos = np.cumsum(np.concatenate([rng.uniform(0, L, (1, N, 3)),
                                    rng.normal(0, 0.4, (T - 1, N, 3))]), axis=0)
    types = rng.integers(0, 3, N).astype(np.int32) * 4 + 1
    if tric:
        box = np.tile([0, L, 0, L, 0, L, 0.3 * L, 0.2 * L, 0.1 * L], (T, 1)).astype(float)
        fmt = ref.BoxFormat.LammpsTriclinic
    else:
        box = np.tile([0, L, 0, L * 1.1, 0, L * 0.9], (T, 1)).astype(float)
        fmt = ref.BoxFormat.LammpsOrtho
    nthreads = int(rng.integers(1, 5))
    skip = int(rng.integers(1, 6))
    every = int(rng.integers(1, 3))
    tmax = int(rng.integers(0, 6))
    n = int(rng.integers(3, T // 2))
    leff = n if (n < tmax or tmax == 0) else tmax
    primo = int(rng.integers(0, max(1, T + 1 - leff - n)))
    rmin = float(rng.choice([0.0, 0.3]))
    rmax = float(rng.uniform(2.0, 4.5))
    nbin = int(rng.integers(5, 80))
    tr = ref.Trajectory(pos, np.zeros_like(pos), types, box, fmt, wrap, False)
    g = ref.Gofrt(tr, rmin, rmax, nbin, tmax, nthreads, skip, every, False)
    g.reset(n)
    g.calculate(primo)
    want = np.array(g, copy=True)
    c = oracle_mod.gofrt_counts(tr.internal_positions(), tr.internal_boxes(),
                                tr.internal_type_ids(), tr.get_ntypes(), rmin, rmax, nbin, tmax,
                                nthreads, skip, every, n, primo, tric=tric, per_thread=True)
    got = oracle_mod.fold_buffer(c, oracle_mod.incr(n, skip))
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


@pytest.mark.parametrize("seed", range(6))
def test_random_msd_bit_exact(ref, oracle_mod, seed):
    """The MSD restatement against the reference's MeanSquareDisplacement:
    random trajectories, box formats, origin strides, lag caps, thread counts
    and both centre-of-mass options; running means identical to the bit."""
    rng = np.random.default_rng(100 + seed)
    N = int(rng.integers(5, 50))
    T = int(rng.integers(15, 40))
    L = float(rng.uniform(4, 9))
    tric = bool(seed % 2)
    wrap = bool((seed // 2) % 2) or tric
    pos = np.cumsum(np.concatenate([rng.uniform(0, L, (1, N, 3)),
                                    rng.normal(0, 0.5, (T - 1, N, 3))]), axis=0)
    types = rng.integers(0, 3, N).astype(np.int32)
    if tric:
        box = np.tile([0, L, 0, L, 0, L, 0.3 * L, 0.2 * L, 0.1 * L], (T, 1)).astype(float)
        fmt = ref.BoxFormat.LammpsTriclinic
    else:
        box = np.tile([0, L, 0, L, 0, L], (T, 1)).astype(float)
        fmt = ref.BoxFormat.LammpsOrtho
    skip = int(rng.integers(1, 5))
    tmax = int(rng.integers(0, 8))
    nthreads = int(rng.integers(1, 4))
    cm_msd, cm_self = bool(rng.integers(0, 2)), bool(rng.integers(0, 2))
    n = int(rng.integers(3, T // 2))
    leff = n if (n < tmax or tmax == 0) else tmax
    primo = int(rng.integers(0, max(1, T + 1 - leff - n)))
    tr = ref.Trajectory(pos, np.zeros_like(pos), types, box, fmt, wrap, False)
    m = ref.MeanSquareDisplacement(tr, skip, tmax, nthreads, cm_msd, cm_self, False)
    m.reset(n)
    m.calculate(primo)
    want = np.array(m, copy=True)
    got = oracle_mod.msd(tr.internal_positions(), tr.internal_type_ids(), tr.get_ntypes(), skip,
                         tmax, n, primo, cm_msd, cm_self,
                         cm=oracle_mod.centres(pos, tr.internal_type_ids(), tr.get_ntypes()))
    assert got.shape == want.shape
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("seed", range(6))
def test_random_neighbours_bit_exact(ref, oracle_mod, seed):
    """The neighbour-list restatement against the reference's Neighbours: sizes,
    indices and {r, x, y, z} rows of every list, sorted or not, or the
    reference's overflow message."""
    rng = np.random.default_rng(200 + seed)
    N = int(rng.integers(20, 90))
    T = 3
    L = float(rng.uniform(6, 10))
    tric = bool(seed % 2)
    pos = np.cumsum(np.concatenate([rng.uniform(0, L, (1, N, 3)),
                                    rng.normal(0, 0.3, (T - 1, N, 3))]), axis=0)
    if seed % 3 == 2:
        pos = pos + L * rng.integers(-3, 4, (1, N, 3))  # far outside the box
    types = rng.integers(0, 2, N).astype(np.int32) * 3
    if tric:
        box = np.tile([0, L, 0, L, 0, L, 0.3 * L, 0.2 * L, 0.1 * L], (T, 1)).astype(float)
        fmt, wrap = ref.BoxFormat.LammpsTriclinic, True
    else:
        box = np.tile([0, L, 0, L, 0, L], (T, 1)).astype(float)
        fmt, wrap = ref.BoxFormat.LammpsOrtho, False
    tr = ref.Trajectory(pos, np.zeros_like(pos), types, box, fmt, wrap, False)
    nt = int(tr.get_ntypes())
    cap = int(rng.choice([4, 40]))
    spec = [(cap, float(rng.uniform(1.5, 2.6)) ** 2, 2.8 ** 2) for _ in range(nt)]
    ts, sort = int(rng.integers(0, T)), bool(seed % 2 == 0)
    nb = ref.Neighbours(tr, spec)
    try:
        nb.calculate_neigh(ts, sort)
        err = None
    except RuntimeError as e:
        err = str(e)
    if err is not None:
        with pytest.raises(oracle_mod.TooManyNeighbours) as eo:
            oracle_mod.neighbours(tr.internal_positions(), tr.internal_boxes(),
                                  tr.internal_type_ids(), nt, ts, spec, sort)
        assert str(eo.value) == err
        return
    o = oracle_mod.neighbours(tr.internal_positions(), tr.internal_boxes(),
                              tr.internal_type_ids(), nt, ts, spec, sort)
    for a in range(N):
        for k in range(nt):
            idx = np.asarray(nb.get_neigh_idx(a, k)).astype(np.int64)
            np.testing.assert_array_equal(o.idx(a, k), idx)
            np.testing.assert_array_equal(o.r(a, k), nb.get_neigh(a, k))
