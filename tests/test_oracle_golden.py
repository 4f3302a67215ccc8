"""The C restatement (oracle/gofr_oracle.c) against fixtures produced by the
reference's own Gofrt build (tests/golden/make_golden.py).

Like the reference's tests/test_gofrt.py and tests/src/test_lammps2020.cpp:
construct Gofrt with a thread count, reset(n), calculate(primo), compare the
whole result buffer -- here bit for bit, including the reference's
per-thread fold of incr.
"""
import numpy as np
import pytest

import golden_util as gu

NAMES = gu.names()


def test_fixtures_present():
    assert len(NAMES) >= 9


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_reference_buffer(oracle_mod, name):
    g = gu.load(name)
    m = g["meta"]
    c = oracle_mod.gofrt_counts(g["internal_positions"], g["internal_boxes"],
                                g["internal_type_ids"], m["ntypes"], m["rmin"], m["rmax"],
                                m["nbin"], m["tmax"], m["nthreads"], m["skip"], m["every"],
                                m["ntimesteps"], m["primo"], tric=m["triclinic"], per_thread=True)
    buf = oracle_mod.fold_buffer(c, oracle_mod.incr(m["ntimesteps"], m["skip"]))
    ref = g["ref_buffer"]
    assert buf.shape == ref.shape
    assert np.array_equal(buf.view(np.uint64), ref.view(np.uint64))
    # counts are recoverable from the reference buffer as rint(v / incr)
    tot = c.sum(axis=0)
    assert np.array_equal(np.rint(ref / gu.incr(m)).astype(np.uint64), tot)


@pytest.mark.parametrize("name", [n for n in NAMES])
def test_oracle_preprocessing_matches_reference(oracle_mod, name):
    """Box conversion and pbc wrap of the reference's Trajectory_numpy."""
    g = gu.load(name)
    m = g["meta"]
    if m["box_format"] == "CellVectors":
        pytest.skip("cell-vector input: internal buffers come from the reference's QR")
    ib = oracle_mod.lammps_to_internal(g["box"])
    assert np.array_equal(ib, g["internal_boxes"])
    if m["wrap"]:
        ip = oracle_mod.pbc_wrap(g["positions"], ib, m["triclinic"])
    else:
        ip = g["positions"]
    assert np.array_equal(ip, g["internal_positions"])


def test_kat_bin_edges(oracle_mod):
    """Known answers pinned by the fixture: d=0.2999999999 (dr=0.1) is bin 3
    because the quotient is rounded to float; d=0.9999999999 with rmax=1 is
    dropped; |dx| == l/2 is not wrapped (d=5 stays 5 and is out of range)."""
    g = gu.load("kat_bin_edges")
    buf = g["ref_buffer"][0]
    counts = np.rint(buf / gu.incr(g["meta"])).astype(int)
    distinct = counts[:3].sum(axis=0)   # channels of distinct pairs
    assert distinct[3] == 2            # 0.2999999999
    assert distinct[4] == 2            # 0.45
    assert distinct[0] == 2            # 0.05
    assert distinct[1] == 2            # 0.1 (as 1.1 - 1.0)
    assert distinct[7] == 2            # 0.7000000001
    assert distinct.sum() == 10        # 0.9999999999 and 5.0 dropped
    assert oracle_mod.bin_of(0.2999999999 ** 2, 0.0, 1.0, 10) == 3
    assert oracle_mod.bin_of(0.9999999999 ** 2, 0.0, 1.0, 10) == -1
    xi, xj = np.array([0.0, 0.0, 0.0]), np.array([5.0, 0.0, 0.0])
    assert oracle_mod.d2(xi, xj, [0, 0, 0, 5.0, 5.0, 5.0], False) == 25.0


def test_self_channel_lag0_all_in_bin0():
    """rmin=0, lag 0: every atom pairs with itself at distance 0 (the reference
    CLI golden tests/data/cli/pair_corr_t shows this as the bin-0 self column)."""
    g = gu.load("self_lag0")
    m = g["meta"]
    counts = np.rint(g["ref_buffer"] / gu.incr(m)).astype(int)
    nt = m["ntypes"]
    half = nt * (nt + 1) // 2
    n_orig = -(-m["ntimesteps"] // m["skip"])
    assert counts[0, half:, 0].sum() == n_orig * g["positions"].shape[1]
    assert counts[0, half:, 1:].sum() == 0


def test_result_layout_matches_reference_contract():
    """shape (leff, ntypes(ntypes+1), nbin) of lib/src/gofrt.cpp:65-71."""
    for name in NAMES:
        g = gu.load(name)
        m = g["meta"]
        leff = m["ntimesteps"] if (m["ntimesteps"] < m["tmax"] or m["tmax"] == 0) else m["tmax"]
        assert g["ref_buffer"].shape == (leff, m["ntypes"] * (m["ntypes"] + 1), m["nbin"])


def test_fma_contraction_is_off(oracle_mod):
    """The oracle must use separate multiply and add, as the reference's x86-64
    build does: for these values x*x + y*y rounded twice (5.052844223689515)
    differs from fma(y, y, x*x) (5.052844223689514)."""
    from fractions import Fraction
    x, y = 1.4453871940548013, 1.7215400323407826
    sep = (x * x) + (y * y)
    fused = float(Fraction(x * x) + Fraction(y) * Fraction(y))
    assert sep != fused
    xi, xj = np.array([x, y, 0.0]), np.zeros(3)
    assert oracle_mod.d2(xi, xj, [0, 0, 0, 10.0, 10.0, 10.0], False) == sep
