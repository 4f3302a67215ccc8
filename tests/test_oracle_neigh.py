"""The neighbour-list restatement in oracle/gofr_oracle.c against fixtures
produced by the reference's own Neighbours (tests/golden/neigh, generated by
tests/golden/make_golden_neigh.py): list sizes, ascending or distance-sorted
indices, {r, x, y, z} rows and SANN counts bit for bit, and the reference's
"Too many neighbours in shell!" error with its message."""
import numpy as np
import pytest

import golden_util as gu

NAMES = gu.neigh_names()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_neighbours_match_reference(oracle_mod, name):
    d = gu.load_neigh(name)
    m = d["meta"]
    spec = [tuple(s) for s in m["spec"]]
    args = (d["internal_positions"], d["internal_boxes"], d["internal_type_ids"], m["ntypes"],
            m["timestep"], spec, m["sort"])
    if m["error"]:
        with pytest.raises(RuntimeError) as e:
            oracle_mod.neighbours(*args)
        assert str(e.value) == m["error"]
        return
    o = oracle_mod.neighbours(*args)
    ent = gu.neigh_entries(d)
    N, nt = d["sizes"].shape
    for a in range(N):
        for k in range(nt):
            idx, rows = ent[a, k]
            assert o.size(a, k) == len(idx)
            np.testing.assert_array_equal(o.idx(a, k).astype(np.int64), idx)
            np.testing.assert_array_equal(o.r(a, k), rows)
            if m["sort"]:
                assert o.sann_n(a, k) == d["sann"][a, k]


def test_fixture_set_present():
    assert len(NAMES) >= 6
