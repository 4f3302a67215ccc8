"""Generates tests/golden/neigh/*.npz with the reference's own Neighbours build.

Run where the analisi source tree is present (it builds oracle/_ref with
oracle/build_ref.sh if needed):

    python tests/golden/make_golden_neigh.py [--ref /path/to/analisi]

Each fixture holds a small seeded input (raw arrays as a user passes them to
pyanalisi.Trajectory), the Neighbours list spec, the frame and sort flag of
calculate_neigh, and what the reference computed: for every (atom, neighbour
type) the list size, indices, {r, x, y, z} rows and the SANN count, or the
message of its "Too many neighbours in shell!" error; plus its internal
positions, boxes and type ids.  The reference has no neighbour-list test data;
these seeded cases make its Python binding's calls (pyanalisi.cpp:196-236).
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import load_ref, walk  # noqa: E402


def cases():
    """(name, pos, types, box, box format, wrap, spec, timestep, sort)."""
    out = []
    rng = np.random.default_rng(4242)
    # 1. orthorhombic, two labels, different cutoffs per type, sorted
    N, T, L = 90, 3, 7.0
    pos = walk(rng, N, T, L, 0.2)
    types = rng.choice([2, 5], N).astype(np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L], (T, 1))
    out.append(("neigh_ortho_sorted", pos, types, box, "LammpsOrtho", False,
                [(40, 2.1 ** 2, 2.6 ** 2), (40, 2.4 ** 2, 2.9 ** 2)], 1, True))
    # 2. atoms far outside the box (iterated minimum image), three labels, unsorted
    pos = walk(rng, N, T, L, 0.3) + L * rng.integers(-3, 4, (1, N, 3))
    types = rng.choice([9, 1, 4], N).astype(np.int32)
    out.append(("neigh_far_unsorted", pos, types, box, "LammpsOrtho", False,
                [(40, 1.9 ** 2, 2.5 ** 2), (40, 2.2 ** 2, 2.5 ** 2), (40, 2.0 ** 2, 2.5 ** 2)],
                2, False))
    # 3. triclinic LAMMPS box, wrapped, sorted
    pos = walk(rng, N, T, L, 0.2)
    types = rng.choice([0, 1], N).astype(np.int32)
    boxt = np.tile([0.0, L, 0.0, L, 0.0, L, 0.9, 0.5, 0.3], (T, 1))
    out.append(("neigh_triclinic", pos, types, boxt, "LammpsTriclinic", True,
                [(40, 2.3 ** 2, 2.8 ** 2), (40, 2.3 ** 2, 2.8 ** 2)], 0, True))
    # 4. non-diagonal cell vectors (rotated internally), sorted
    N, T = 70, 2
    pos = walk(rng, N, T, 6.5, 0.2)
    types = rng.choice([0, 1], N).astype(np.int32)
    cell = np.array([[6.5, 1.2, 0.4], [0.0, 6.5, 0.7], [0.0, 0.0, 6.5]])
    out.append(("neigh_rotated", pos, types, np.tile(cell, (T, 1, 1)), "CellVectors", False,
                [(40, 2.2 ** 2, 2.7 ** 2), (40, 2.0 ** 2, 2.7 ** 2)], 1, True))
    # 5. a list fills up: the reference's error
    N, T, L = 60, 2, 6.0
    pos = walk(rng, N, T, L, 0.2)
    types = rng.choice([0, 1], N).astype(np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L], (T, 1))
    out.append(("neigh_overflow", pos, types, box, "LammpsOrtho", False,
                [(4, 2.6 ** 2, 3.0 ** 2), (6, 2.6 ** 2, 3.0 ** 2)], 0, True))
    # 6. lists exactly full but never overflowing: capacity = the largest size
    out.append(("neigh_exactly_full", pos, types, box, "LammpsOrtho", False,
                [(None, 1.6 ** 2, 2.0 ** 2), (None, 1.8 ** 2, 2.0 ** 2)], 1, True))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ANALISI_REF"),
                    required="ANALISI_REF" not in os.environ,
                    help="root of the reference tree (or set ANALISI_REF)")
    args = ap.parse_args()
    pa = load_ref(args.ref)
    outdir = os.path.join(HERE, "neigh")
    os.makedirs(outdir, exist_ok=True)
    for name, pos, types, box, fmt, wrap, spec, ts, sort in cases():
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        box = np.ascontiguousarray(box, dtype=np.float64)
        tr = pa.Trajectory(pos, np.zeros_like(pos), types, box, getattr(pa.BoxFormat, fmt), wrap,
                           False)
        nt = int(tr.get_ntypes())
        N = pos.shape[1]
        if any(s[0] is None for s in spec):
            # capacity = the largest list of that type, found with roomy lists
            big = pa.Neighbours(tr, [(N, s[1], s[2]) for s in spec])
            big.calculate_neigh(ts, sort)
            spec = [(max(len(big.get_neigh_idx(a, k)) for a in range(N)), s[1], s[2])
                    for k, s in enumerate(spec)]
        nb = pa.Neighbours(tr, spec)
        err = ""
        sizes = np.zeros((N, nt), dtype=np.int64)
        sann = np.zeros((N, nt), dtype=np.int64)
        idx, rows = [], []
        try:
            nb.calculate_neigh(ts, sort)
            for a in range(N):
                for k in range(nt):
                    i = nb.get_neigh_idx(a, k)
                    sizes[a, k] = len(i)
                    idx.append(np.asarray(i, dtype=np.int64))
                    rows.append(nb.get_neigh(a, k).copy())
                    if sort:
                        sann[a, k] = len(nb.get_sann_idx(a, k))
        except RuntimeError as e:
            err = str(e)
        meta = dict(name=name, box_format=fmt, wrap=wrap, spec=[list(s) for s in spec],
                    timestep=ts, sort=sort, ntypes=nt, error=err)
        np.savez_compressed(
            os.path.join(outdir, name + ".npz"), positions=pos, types=types, box=box,
            sizes=sizes, sann=sann,
            idx=np.concatenate(idx) if idx else np.zeros(0, np.int64),
            rows=np.concatenate(rows) if rows else np.zeros((0, 4)),
            internal_positions=tr.internal_positions().copy(),
            internal_boxes=tr.internal_boxes().copy(),
            internal_type_ids=tr.internal_type_ids().copy(), meta=json.dumps(meta))
        print(f"{name}: spec {spec}, total {int(sizes.sum())} entries, error {err!r}")


if __name__ == "__main__":
    main()
