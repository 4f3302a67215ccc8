"""Batched trajectories in one persistent launch (gofr_batch_set /
gofr_batch_run): every member's counts equal the oracle's, with and without
the CUDA graph, on repeated runs.  Members are uneven in atoms, frames, types,
box size (small boxes use the wrap-decision check) and cell shape."""
import numpy as np
import pytest

from analisi_gb300 import workloads

pytestmark = pytest.mark.gpu

MEMBERS = [
    # seed, N, T, L, sigma, counts, tric, wrap, params
    (51, 700, 14, 19.0, 0.1, [400, 300], False, False,
     dict(rmin=0.0, rmax=6.0, nbin=60, tmax=4, skip=3, every=1, ntimesteps=9, primo=0)),
    (52, 90, 20, 6.0, 0.3, [45, 45], False, False,          # rmax > l/2: wrap check
     dict(rmin=0.0, rmax=5.0, nbin=50, tmax=5, skip=2, every=1, ntimesteps=12, primo=1)),
    (53, 1300, 8, 24.0, 0.1, [1000, 200, 100], False, False,
     dict(rmin=0.2, rmax=7.0, nbin=70, tmax=2, skip=2, every=1, ntimesteps=5, primo=0)),
    (54, 300, 12, 14.0, 0.2, [300], True, True,             # triclinic member
     dict(rmin=0.0, rmax=5.0, nbin=40, tmax=3, skip=2, every=2, ntimesteps=8, primo=0)),
    (55, 40, 30, 4.0, 0.3, [10, 10, 10, 10], False, False,  # tiny box, 4 types
     dict(rmin=0.0, rmax=3.0, nbin=30, tmax=6, skip=5, every=1, ntimesteps=20, primo=2)),
]


def _oracle(oracle_mod, w):
    p = w["params"]
    return oracle_mod.gofrt_counts(w["positions"], w["boxes"], w["type_ids"], w["ntypes"],
                                   p["rmin"], p["rmax"], p["nbin"], p["tmax"], 1, p["skip"],
                                   p["every"], p["ntimesteps"], p["primo"], tric=w["triclinic"])


@pytest.fixture(scope="module")
def members():
    return [workloads.small_case(s, N, T, L, sg, c, tric=tr, wrap_into_cell=wr, **p)
            for (s, N, T, L, sg, c, tr, wr, p) in MEMBERS]


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_oracle(built_engine, oracle_mod, members, use_graph):
    from analisi_gb300 import engine
    trajs = []
    for w in members:
        p = w["params"]
        trajs.append(dict(positions=w["positions"], boxes=w["boxes"], type_ids=w["type_ids"],
                          ntypes=w["ntypes"],
                          params=engine.make_params(p["rmin"], p["rmax"], p["nbin"], p["tmax"],
                                                    p["skip"], p["every"], p["ntimesteps"],
                                                    p["primo"])))
    refs = [_oracle(oracle_mod, w) for w in members]
    with engine.Engine(0) as e:
        e.batch_set(trajs)
        for rep in range(2):
            outs = e.batch_run(use_graph=use_graph)
            for k, (got, ref) in enumerate(zip(outs, refs)):
                assert got.shape == ref.shape, k
                np.testing.assert_array_equal(got, ref, err_msg=f"member {k} run {rep}")
        st = e.stats()
        assert st["pairs"] == sum(workloads.pairs_of(w["positions"].shape[1], w["params"])
                                  for w in members)


CELL_MEMBERS = [
    # large enough boxes for cell lists (orthorhombic, constant), plus a small member
    (56, 4000, 8, 34.2, 0.2, [3000, 1000], False, False,
     dict(rmin=0.0, rmax=5.0, nbin=50, tmax=2, skip=2, every=1, ntimesteps=5, primo=1)),
    (57, 3000, 7, 31.0, 0.2, [3000], False, False,
     dict(rmin=0.5, rmax=4.5, nbin=40, tmax=3, skip=3, every=1, ntimesteps=4, primo=0)),
    (58, 5000, 6, 36.8, 0.1, [2000, 2000, 1000], False, False,
     dict(rmin=0.0, rmax=5.5, nbin=55, tmax=2, skip=1, every=1, ntimesteps=3, primo=0)),
    (59, 200, 10, 12.0, 0.2, [150, 50], False, False,
     dict(rmin=0.0, rmax=4.0, nbin=40, tmax=3, skip=2, every=1, ntimesteps=6, primo=0)),
]


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_with_cell_members(built_engine, oracle_mod, use_graph):
    """Members the planner runs with cell lists share one multi-trajectory
    cell-list launch next to the all-pairs one; counts stay the oracle's."""
    from analisi_gb300 import engine
    mem = [workloads.small_case(s, N, T, L, sg, c, tric=tr, wrap_into_cell=wr, **p)
           for (s, N, T, L, sg, c, tr, wr, p) in CELL_MEMBERS]
    trajs = []
    for w in mem:
        p = w["params"]
        trajs.append(dict(positions=w["positions"], boxes=w["boxes"], type_ids=w["type_ids"],
                          ntypes=w["ntypes"],
                          params=engine.make_params(p["rmin"], p["rmax"], p["nbin"], p["tmax"],
                                                    p["skip"], p["every"], p["ntimesteps"],
                                                    p["primo"])))
    refs = [_oracle(oracle_mod, w) for w in mem]
    with engine.Engine(0) as e:
        e.batch_set(trajs)
        for rep in range(2):
            outs = e.batch_run(use_graph=use_graph)
            for k, (got, ref) in enumerate(zip(outs, refs)):
                np.testing.assert_array_equal(got, ref, err_msg=f"member {k} run {rep}")
        st = e.stats()
        assert st["evaluated"] < st["pairs"]  # some members ran with cell lists
