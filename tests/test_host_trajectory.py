"""The drop-in Python module's Trajectory (analisi_gb300/host/trajectory.cpp)
against the reference's own preprocessing, captured in tests/golden/: box
conversion, pbc wrap, the QR rotation of non-diagonal cell vectors, dense type
ids -- all bit for bit.  Needs no GPU (the module only touches the device in
Gofrt.calculate)."""
import numpy as np
import pytest

import golden_util as gu


@pytest.fixture(scope="module")
def pa(built_engine):
    from analisi_gb300 import build
    build.build_host()
    import analisi_gb300
    return analisi_gb300.load_pyanalisi()


@pytest.mark.parametrize("name", gu.names())
def test_internal_buffers_match_reference(pa, name):
    g = gu.load(name)
    m = g["meta"]
    t = pa.Trajectory(g["positions"], np.zeros_like(g["positions"]), g["types"], g["box"],
                      getattr(pa.BoxFormat, m["box_format"]), m["wrap"], False)
    assert np.array_equal(t.get_positions_copy(), g["internal_positions"])
    assert np.array_equal(t.get_box_copy(), g["internal_boxes"])
    assert np.array_equal(t.get_type_ids(), g["internal_type_ids"])
    assert t.get_ntypes() == m["ntypes"]
    assert t.is_triclinic() == m["triclinic"]


def test_negative_type_labels_sort_as_unsigned(pa):
    """The reference keeps raw labels in a std::vector<unsigned int>, so -1 sorts
    after 7 (lib/src/basetrajectory.cpp:60-79)."""
    pos = np.random.default_rng(0).uniform(0, 5, (2, 4, 3))
    t = pa.Trajectory(pos, np.zeros_like(pos), np.array([7, -1, 3, 7], dtype=np.int32),
                      np.tile([0, 5.0, 0, 5.0, 0, 5.0], (2, 1)), pa.BoxFormat.LammpsOrtho,
                      False, False)
    assert list(t.get_type_ids()) == [1, 2, 0, 1]


def test_rotation_matrix_saved(pa):
    g = gu.load("cellvec_tric")
    t = pa.Trajectory(g["positions"], np.zeros_like(g["positions"]), g["types"], g["box"],
                      pa.BoxFormat.CellVectors, False, True)
    r = t.get_rotation_matrix()
    assert r.shape == (g["positions"].shape[0], 3, 3)
    q = r[0].T
    assert np.allclose(q @ q.T, np.eye(3), atol=1e-14)


@pytest.mark.parametrize("bad,msg", [
    ("pos2d", "Wrong number of dimension of position array"),
    ("types_float", "Format of types array should be int"),
    ("box_shape", "must be (:, 6) for orthogonal lammps cell format"),
    ("strided", "Unsupported stride in pos array"),
])
def test_argument_errors_match_reference(pa, bad, msg):
    pos = np.zeros((3, 4, 3))
    vel = np.zeros_like(pos)
    types = np.zeros(4, dtype=np.int32)
    box = np.tile([0, 5.0, 0, 5.0, 0, 5.0], (3, 1))
    if bad == "pos2d":
        pos = pos[0]
    elif bad == "types_float":
        types = types.astype(np.float64)
    elif bad == "box_shape":
        box = box[:, :5].copy()
    elif bad == "strided":
        pos = np.zeros((3, 8, 3))[:, ::2]
        vel = np.zeros((3, 4, 3))
    with pytest.raises(RuntimeError, match=msg.replace("(", r"\(").replace(")", r"\)")):
        pa.Trajectory(pos, vel, types, box, pa.BoxFormat.LammpsOrtho, False, False)


@pytest.mark.parametrize("name", gu.msd_names())
def test_centres_of_mass_match_reference(pa, name):
    """Per-type centres of mass, from the caller's positions before wrapping or
    rotation, bit for bit (the reference's positions_cm)."""
    g = gu.load_msd(name)
    m = g["meta"]
    t = pa.Trajectory(g["positions"], np.zeros_like(g["positions"]), g["types"], g["box"],
                      getattr(pa.BoxFormat, m["box_format"]), m["wrap"], False)
    assert np.array_equal(t.get_positions_copy(), g["internal_positions"])
    assert np.array_equal(t.get_type_ids(), g["internal_type_ids"])
    assert np.array_equal(t.get_centres_copy(), g["internal_centres"])
