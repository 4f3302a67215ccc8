"""The planner's choices on the host (gofr_plan_query: the same code gofr_run
plans with, no GPU, tuner cache not consulted) for the five Gofrt workloads
and the edge cases: the warp-streamed cell-list kernel on the 16k-, 32k-
(triclinic) and 131k-atom boxes, the all-pairs kernel on the small box and on
the batch's smallest member (with its per-pair wrap check), a sparse box
(more cells than atoms allowed), plain FP64 on request and for bin maps the
FP32 path cannot certify, and forced cell-list kernels the box cannot take."""
import math

import pytest

from analisi_gb300 import engine

F32, F64, CELL, CELLW = 1, 2, 3, 5


def cube(L):
    return [0.0, 0.0, 0.0, L / 2, L / 2, L / 2]


def plan(box, tric, lo, hi, N, nt, *args, kernel="auto"):
    return engine.plan_query(box, tric, lo, hi, N, nt, engine.make_params(*args, kernel=kernel))


def test_16k_atom_workload_takes_single_cell_warp_blocks(built_engine):
    L = (16384 / 0.1) ** (1 / 3)
    p = plan(cube(L), False, [-5.0] * 3, [L + 5.0] * 3, 16384, 3, 0.0, 12.0, 400, 200, 4, 1,
             1800, 0)
    assert p == {"kernel": CELLW, "reach": 2, "cells": (9, 9, 9), "block": (1, 1, 1),
                 "cta_warps": 16, "wrapcheck": False}


def test_131k_atom_workload_takes_reach_three(built_engine):
    L = (131072 / 0.1) ** (1 / 3)
    p = plan(cube(L), False, [-5.0] * 3, [L + 5.0] * 3, 131072, 4, 0.0, 10.0, 250, 50, 10, 1,
             450, 0)
    assert (p["kernel"], p["reach"], p["cells"], p["block"]) == (CELLW, 3, (32, 32, 32), (2, 2, 2))


def test_triclinic_workload_takes_the_warp_kernel(built_engine):
    L = 70.0
    box = cube(L) + [0.3 * L, 0.2 * L, 0.1 * L]
    p = plan(box, True, [0.0] * 3, [1.5 * L, 1.1 * L, L], 32768, 2, 0.0, 15.0, 500, 100, 5, 1,
             900, 0)
    assert p["kernel"] == CELLW and p["reach"] >= 1 and not p["wrapcheck"]
    # forcing the block cell-list kernel in a triclinic box is refused
    with pytest.raises(engine.GofrError) as err:
        plan(box, True, [0.0] * 3, [1.5 * L, 1.1 * L, L], 32768, 2, 0.0, 15.0, 500, 100, 5, 1,
             900, 0, kernel="cell")
    assert err.value.code == -7


def test_small_boxes_stay_on_all_pairs(built_engine):
    # the 1000-atom box: the neighbourhood would be most of the box
    p = plan(cube(22.0), False, [-2.0] * 3, [24.0] * 3, 1000, 2, 0.7, 3.5, 200, 20, 10, 1, 180, 0)
    assert p["kernel"] == F32 and not p["wrapcheck"]
    # the batch's smallest member: L/2 < rmax, all pairs with the per-pair wrap check
    L = (256 / 0.1) ** (1 / 3)
    p = plan(cube(L), False, [-2.0] * 3, [L + 2.0] * 3, 256, 2, 0.0, 10.0, 300, 100, 5, 1, 500, 0)
    assert p["kernel"] == F32 and p["wrapcheck"]
    with pytest.raises(engine.GofrError):
        plan(cube(L), False, [-2.0] * 3, [L + 2.0] * 3, 256, 2, 0.0, 10.0, 300, 100, 5, 1, 500,
             0, kernel="cellw")


def test_sparse_box_over_the_cell_cap_plans_all_pairs(built_engine):
    p = plan(cube(60.0), False, [0.0] * 3, [60.0] * 3, 60, 2, 0.0, 5.0, 40, 2, 2, 1, 3, 0)
    assert p["kernel"] == F32


def test_fp64_on_request_and_for_uncertifiable_bins(built_engine):
    L = (16384 / 0.1) ** (1 / 3)
    p = plan(cube(L), False, [-5.0] * 3, [L + 5.0] * 3, 16384, 3, 0.0, 12.0, 400, 200, 4, 1,
             1800, 0, kernel="f64")
    assert p["kernel"] == F64
    # rmax <= rmin: the bin map is not monotone, AUTO takes plain FP64
    p = plan(cube(L), False, [-5.0] * 3, [L + 5.0] * 3, 16384, 3, 5.0, 5.0, 10, 2, 1, 1, 3, 0)
    assert p["kernel"] == F64


def test_forced_kernels_are_honoured(built_engine):
    L = (16384 / 0.1) ** (1 / 3)
    args = (0.0, 12.0, 400, 200, 4, 1, 1800, 0)
    assert plan(cube(L), False, [-5.0] * 3, [L + 5.0] * 3, 16384, 3, *args,
                kernel="f32")["kernel"] == F32
    p = plan(cube(L), False, [-5.0] * 3, [L + 5.0] * 3, 16384, 3, *args, kernel="cell")
    assert p["kernel"] == CELL and p["cells"] == (9, 9, 9)
    assert plan(cube(L), False, [-5.0] * 3, [L + 5.0] * 3, 16384, 3, *args,
                kernel="cellw")["kernel"] == CELLW
    with pytest.raises(engine.GofrError):
        plan(cube(L), False, [-5.0] * 3, [L + 5.0] * 3, 16384, 3, *args, kernel=9)
