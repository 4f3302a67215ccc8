"""Neighbour lists on the GPU (gofr_neigh_run, the drop-in pyanalisi.Neighbours)
against the reference's own lists (tests/golden/neigh) and the oracle: sizes,
indices, {r, x, y, z} rows and SANN counts bit for bit (every value is the
reference's FP64 arithmetic), the overflow error with the reference's message,
and a larger triclinic case."""
import numpy as np
import pytest

import golden_util as gu
from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu

NAMES = gu.neigh_names()


@pytest.fixture(scope="module")
def pa(built_engine):
    from analisi_gb300 import build
    build.build_host()
    import analisi_gb300
    return analisi_gb300.load_pyanalisi()


def _compare(get_size, get_idx, get_rows, get_sann, d):
    ent = gu.neigh_entries(d)
    N, nt = d["sizes"].shape
    for a in range(N):
        for k in range(nt):
            idx, rows = ent[a, k]
            assert get_size(a, k) == len(idx), (a, k)
            np.testing.assert_array_equal(np.asarray(get_idx(a, k)).astype(np.int64), idx)
            np.testing.assert_array_equal(get_rows(a, k), rows)
            if d["meta"]["sort"]:
                assert get_sann(a, k) == d["sann"][a, k]


@pytest.mark.parametrize("name", NAMES)
def test_engine_neighbours_match_reference(gpu_engine, name):
    from analisi_gb300 import engine
    d = gu.load_neigh(name)
    m = d["meta"]
    gpu_engine.set_frames(d["internal_positions"], d["internal_boxes"], d["internal_type_ids"],
                          m["ntypes"])
    spec = [tuple(s) for s in m["spec"]]
    if m["error"]:
        with pytest.raises(engine.GofrError) as e:
            gpu_engine.neighbours(m["timestep"], spec, m["sort"])
        assert str(e.value).endswith(m["error"])
        return
    nl = gpu_engine.neighbours(m["timestep"], spec, m["sort"])
    _compare(nl.size, nl.idx, nl.r, nl.sann_n, d)


@pytest.mark.parametrize("name", NAMES)
def test_pyanalisi_neighbours_match_reference(pa, name):
    d = gu.load_neigh(name)
    m = d["meta"]
    t = pa.Trajectory(d["positions"], np.zeros_like(d["positions"]), d["types"], d["box"],
                      getattr(pa.BoxFormat, m["box_format"]), m["wrap"], False)
    nb = pa.Neighbours(t, [tuple(s) for s in m["spec"]])
    if m["error"]:
        with pytest.raises(RuntimeError) as e:
            nb.calculate_neigh(m["timestep"], m["sort"])
        assert str(e.value) == m["error"]
        return
    nb.calculate_neigh(m["timestep"], m["sort"])
    _compare(lambda a, k: len(nb.get_neigh_idx(a, k)), nb.get_neigh_idx, nb.get_neigh,
             lambda a, k: len(nb.get_sann_idx(a, k)), d)
    if m["sort"]:
        a, k = 0, 0
        n = len(nb.get_sann_idx(a, k))
        np.testing.assert_array_equal(nb.get_sann(a, k), nb.get_neigh(a, k)[:n])


@pytest.mark.parametrize("sort", [False, True])
def test_engine_neighbours_match_oracle_triclinic(gpu_engine, oracle_mod, sort):
    """2500 atoms, three types, triclinic cell, coordinates wrapped into it."""
    w = workloads.small_case(81, 2500, 3, 30.0, 0.1, [1200, 800, 500], tric=True,
                             wrap_into_cell=True)
    spec = [(60, 3.1 ** 2, 3.5 ** 2), (60, 2.7 ** 2, 3.5 ** 2), (60, 3.3 ** 2, 3.5 ** 2)]
    o = oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], 3, 1, spec, sort)
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], 3)
    nl = gpu_engine.neighbours(1, spec, sort)
    np.testing.assert_array_equal(nl.list[: len(o.list)][_counted_mask(o)],
                                  o.list[_counted_mask(o)])
    for a in range(0, 2500, 7):
        for k in range(3):
            assert nl.size(a, k) == o.size(a, k)
            np.testing.assert_array_equal(nl.idx(a, k), o.idx(a, k))
            np.testing.assert_array_equal(nl.r(a, k), o.r(a, k))
            if sort:
                assert nl.sann_n(a, k) == o.sann_n(a, k)


def _counted_mask(o):
    """Positions of the list array that hold sizes or counted indices (the
    reference leaves stale entries past a list's size)."""
    mask = np.zeros(len(o.list), dtype=bool)
    for k, n in enumerate(o.nneigh):
        for a in range(o.natoms):
            b = o.loff[k] + a * (n + 1)
            mask[b:b + 1 + o.size(a, k)] = True
    return mask


def test_neighbour_argument_errors(gpu_engine):
    from analisi_gb300 import engine
    w = workloads.small_case(82, 200, 2, 12.0, 0.1, [120, 80])
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], 2)
    with pytest.raises(engine.GofrError, match="each atomic type"):
        gpu_engine.neighbours(0, [(10, 4.0, 5.0)], True)
    with pytest.raises(engine.GofrError, match="outside"):
        gpu_engine.neighbours(5, [(10, 4.0, 5.0), (10, 4.0, 5.0)], True)


def test_engine_neighbours_small_box_fp64_path(gpu_engine, oracle_mod):
    """A cutoff just under half the box: the minimum image of near pairs is not
    certain in FP32, so every pair takes the FP64 path; lists as the oracle's."""
    w = workloads.small_case(83, 300, 2, 6.0, 0.1, [200, 100])
    spec = [(300, 2.99 ** 2, 3.0 ** 2), (300, 2.9 ** 2, 3.0 ** 2)]
    o = oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], 2, 1, spec, True)
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], 2)
    nl = gpu_engine.neighbours(1, spec, True)
    for a in range(300):
        for k in range(2):
            np.testing.assert_array_equal(nl.idx(a, k), o.idx(a, k))
            np.testing.assert_array_equal(nl.r(a, k), o.r(a, k))


def _full_compare(nl, o, sort):
    np.testing.assert_array_equal(nl.list[_counted_mask(o)], o.list[_counted_mask(o)])
    for a in range(o.natoms):
        for k in range(len(o.nneigh)):
            n = o.size(a, k)
            assert nl.size(a, k) == n
            np.testing.assert_array_equal(nl.r(a, k), o.r(a, k))
            if sort:
                assert nl.sann_n(a, k) == o.sann_n(a, k)


@pytest.mark.parametrize("sort", [False, True])
def test_cell_form_matches_oracle_and_all_pairs(gpu_engine, oracle_mod, sort, monkeypatch):
    """Orthorhombic box of 11^3 cells of edge >= the largest cutoff, atoms far
    outside the box (iterated minimum image), a box not at the origin, three
    types: the cell-list form's lists, vectors and SANN counts equal the
    oracle's and the all-pairs form's, bit for bit."""
    L = 40.0
    w = workloads.small_case(84, 4000, 3, L, 0.2, [2000, 1200, 800])
    rng = np.random.default_rng(840)
    shift = np.array([-11.5, 4.25, 7.0])
    w["positions"] = w["positions"] + L * rng.integers(-3, 4, size=(1, 4000, 3)) + shift
    w["boxes"] = w["boxes"].copy()
    w["boxes"][:, 0:3] += shift
    spec = [(50, 3.1 ** 2, 3.6 ** 2), (50, 2.7 ** 2, 3.6 ** 2), (50, 3.5 ** 2, 3.6 ** 2)]
    o = oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], 3, 2, spec, sort)
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], 3)
    monkeypatch.delenv("ANALISI_GB300_NEIGH_KERNEL", raising=False)
    nl = gpu_engine.neighbours(2, spec, sort)
    assert gpu_engine.stats()["kernel_used"] == -2
    _full_compare(nl, o, sort)
    monkeypatch.setenv("ANALISI_GB300_NEIGH_KERNEL", "allpairs")
    nl2 = gpu_engine.neighbours(2, spec, sort)
    assert gpu_engine.stats()["kernel_used"] == -1
    np.testing.assert_array_equal(nl2.list, nl.list)
    np.testing.assert_array_equal(nl2.rpos, nl.rpos)


def test_cell_form_overflow_error_is_the_references(gpu_engine, oracle_mod, monkeypatch):
    """Lists too short for the shell: the cell-list form fills them in the
    reference's order, so the first overflowing pair and the message are the
    reference's."""
    monkeypatch.delenv("ANALISI_GB300_NEIGH_KERNEL", raising=False)
    from analisi_gb300 import engine
    w = workloads.small_case(85, 3000, 2, 36.0, 0.2, [1800, 1200])
    spec = [(5, 3.4 ** 2, 3.6 ** 2), (4, 3.0 ** 2, 3.6 ** 2)]
    with pytest.raises(oracle_mod.TooManyNeighbours) as eo:
        oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], 2, 1, spec, True)
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], 2)
    with pytest.raises(engine.GofrError) as eg:
        gpu_engine.neighbours(1, spec, True)
    assert gpu_engine.stats()["kernel_used"] == -2
    assert str(eg.value).endswith(str(eo.value))


def test_cell_form_dense_neighbourhood_falls_back(gpu_engine, oracle_mod, monkeypatch):
    """A cutoff holding ~400 atoms (more than a warp's survivor buffer): the
    build reruns in the all-pairs form, lists as the oracle's."""
    monkeypatch.delenv("ANALISI_GB300_NEIGH_KERNEL", raising=False)
    w = workloads.small_case(86, 3000, 2, 21.0, 0.1, [1500, 1500])
    spec = [(300, 6.8 ** 2, 7.0 ** 2), (300, 6.5 ** 2, 7.0 ** 2)]
    o = oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], 2, 1, spec, False)
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], 2)
    nl = gpu_engine.neighbours(1, spec, False)
    assert gpu_engine.stats()["kernel_used"] == -1
    _full_compare(nl, o, False)


def test_cell_form_exactly_full_lists(gpu_engine, oracle_mod, monkeypatch):
    """Capacities equal to the largest list of each type: every such list is
    full, so the overflow check runs (in the cell-list form) and must find
    nothing; the lists are the oracle's."""
    monkeypatch.delenv("ANALISI_GB300_NEIGH_KERNEL", raising=False)
    w = workloads.small_case(87, 3000, 2, 36.0, 0.2, [1800, 1200])
    roomy = [(200, 3.4 ** 2, 3.6 ** 2), (200, 3.0 ** 2, 3.6 ** 2)]
    big = oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], 2, 1, roomy, True)
    spec = [(max(big.size(a, k) for a in range(3000)), roomy[k][1], roomy[k][2]) for k in range(2)]
    o = oracle_mod.neighbours(w["positions"], w["boxes"], w["type_ids"], 2, 1, spec, True)
    gpu_engine.set_frames(w["positions"], w["boxes"], w["type_ids"], 2)
    nl = gpu_engine.neighbours(1, spec, True)
    assert gpu_engine.stats()["kernel_used"] == -2
    _full_compare(nl, o, True)
