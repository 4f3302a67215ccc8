"""The MSD restatement in oracle/gofr_oracle.c against fixtures produced by the
reference's own MeanSquareDisplacement (tests/golden/msd, generated by
tests/golden/make_golden_msd.py): bit-identical running means and centres of
mass, including the reference's quirks (centres taken from the caller's
positions before wrapping or rotation; a range error when the trajectory is
too short)."""
import numpy as np
import pytest

import golden_util as gu

NAMES = gu.msd_names()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_msd_matches_reference_bits(oracle_mod, name):
    d = gu.load_msd(name)
    m = d["meta"]
    out = oracle_mod.msd(d["internal_positions"], d["internal_type_ids"], m["ntypes"], m["skip"],
                         m["tmax"], m["ntimesteps"], m["primo"], m["cm_msd"], m["cm_self"],
                         cm=d["internal_centres"])
    assert out.shape == d["ref_buffer"].shape
    np.testing.assert_array_equal(out, d["ref_buffer"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_centres_match_reference_bits(oracle_mod, name):
    """Centres of mass come from the caller's raw positions (not the internal,
    possibly wrapped or rotated, copy)."""
    d = gu.load_msd(name)
    cm = oracle_mod.centres(d["positions"], d["internal_type_ids"], d["meta"]["ntypes"])
    np.testing.assert_array_equal(cm, d["internal_centres"])


def test_oracle_msd_range_error(oracle_mod):
    d = gu.load_msd(NAMES[0])
    m = d["meta"]
    T = d["internal_positions"].shape[0]
    with pytest.raises(RuntimeError, match="too short"):
        oracle_mod.msd(d["internal_positions"], d["internal_type_ids"], m["ntypes"], 1, 5, T - 4,
                       0, cm=d["internal_centres"])


def test_fixture_set_present():
    assert len(NAMES) >= 5
