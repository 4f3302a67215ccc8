"""Test helper: writes analisi's binary trajectory format (classic, classic
triclinic, LAMMPS-2020 headers; several chunks per frame; atoms in any id order)."""
import struct

import numpy as np


def write(path, pos, types, boxes, triclinic=False, new_header=False, nchunk=1, perm=None,
          revision=2):
    T, N = pos.shape[0], pos.shape[1]
    perm = np.arange(N) if perm is None else perm
    with open(path, "wb") as f:
        for t in range(T):
            if new_header:
                magic = b"DUMPATOM"
                f.write(struct.pack("<q", -len(magic)))
                f.write(magic)
                f.write(struct.pack("<ii", 1, revision))
            f.write(struct.pack("<qqi", 100 * t, N, 1 if triclinic else 0))
            f.write(struct.pack("<6i", 0, 0, 0, 0, 0, 0))
            f.write(struct.pack("<6d", *boxes[t, :6]))
            if triclinic:
                f.write(struct.pack("<3d", *boxes[t, 6:9]))
            f.write(struct.pack("<i", 8))
            if new_header and revision > 1:
                unit = b"real"
                f.write(struct.pack("<i", len(unit)))
                f.write(unit)
                f.write(struct.pack("<b", 1))
                f.write(struct.pack("<d", 0.5 * t))
                cols = b"id type xu yu zu vx vy vz"
                f.write(struct.pack("<i", len(cols)))
                f.write(cols)
            f.write(struct.pack("<i", nchunk))
            order = perm if t == 0 else np.roll(perm, t)
            parts = np.array_split(order, nchunk)
            for part in parts:
                f.write(struct.pack("<i", 8 * len(part)))
                for a in part:
                    rec = [float(a + 1), float(types[a]), *pos[t, a], 0.0, 0.0, 0.0]
                    f.write(struct.pack("<8d", *rec))
