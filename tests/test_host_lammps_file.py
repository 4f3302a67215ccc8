"""Reader of analisi's binary trajectories (the CLI input): header kinds,
chunks and the first-frame atom order (lib/src/trajectory.cpp:630-660)."""
import numpy as np
import pytest

import lammps_writer


@pytest.fixture(scope="module")
def pa(built_engine):
    from analisi_gb300 import build
    build.build_host()
    import analisi_gb300
    return analisi_gb300.load_pyanalisi()


@pytest.mark.parametrize("triclinic,new_header,nchunk", [(False, False, 1), (True, False, 3),
                                                         (False, True, 2), (True, True, 1)])
def test_read_back(pa, tmp_path, triclinic, new_header, nchunk):
    rng = np.random.default_rng(5)
    T, N = 4, 11
    pos = rng.uniform(-2, 9, (T, N, 3))
    types = rng.integers(1, 4, N).astype(np.int32)
    row = [0, 8.0, -1, 7.5, 0.5, 9.0] + ([1.0, 0.5, -0.3] if triclinic else [])
    boxes = np.tile(row, (T, 1)).astype(float)
    perm = rng.permutation(N)
    p = str(tmp_path / "t.bin")
    lammps_writer.write(p, pos, types, boxes, triclinic, new_header, nchunk, perm)
    d = pa.read_lammps_binary(p)
    # atoms are indexed in the order they appear in the first frame
    assert np.array_equal(d["positions"], pos[:, perm])
    assert np.array_equal(d["types"], types[perm])
    assert np.array_equal(d["boxes"], boxes)
    assert d["triclinic"] == triclinic
    assert list(d["timesteps"]) == [0, 100, 200, 300]


def test_bad_atom_record_size(pa, tmp_path):
    import struct
    p = tmp_path / "bad.bin"
    with open(p, "wb") as f:
        f.write(struct.pack("<qqi", 0, 1, 0) + struct.pack("<6i", *[0] * 6))
        f.write(struct.pack("<6d", 0, 1, 0, 1, 0, 1) + struct.pack("<ii", 7, 1))
    with pytest.raises(RuntimeError, match="does not have 8 numbers per atom"):
        pa.read_lammps_binary(str(p))
