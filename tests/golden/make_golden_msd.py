"""Generates tests/golden/msd/*.npz with the reference's own MSD build.

Run where the analisi source tree is present (it builds oracle/_ref with
oracle/build_ref.sh if needed):

    python tests/golden/make_golden_msd.py [--ref /path/to/analisi]

Each fixture holds a small seeded input (raw arrays as a user passes them to
pyanalisi.Trajectory), the MeanSquareDisplacement arguments, and what the
reference computed: its result buffer [leff][f_cm][ntypes] and its internal
positions, type ids and per-type centres of mass.  The reference's own MSD
regression input is not available (.MISSING_LARGE_BLOBS), so these seeded
cases stand in for it; they make the calls of the reference's tests/test_msd.py
(MeanSquareDisplacement(traj, skip, tmax, nthreads, cm_msd, cm_self, debug),
reset(n), calculate(primo)).
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
    """(name, pos, types, box, box format, wrap, MSD args, reset n, primo)."""
    out = []
    rng = np.random.default_rng(31337)
    # 1. orthorhombic box, two raw labels, plain MSD, primo > 0, skip not dividing n
    N, T, L = 40, 26, 8.0
    pos = walk(rng, N, T, L, 0.35)
    types = rng.choice([4, 2], N).astype(np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L], (T, 1))
    out.append(("msd_ortho", pos, types, box, "LammpsOrtho", False,
                dict(skip=3, tmax=6, nthreads=2, cm_msd=False, cm_self=False), 13, 2))
    # 2. both centre-of-mass options, three labels, tmax 0 (leff = n)
    pos = walk(rng, N, T, L, 0.5)
    types = rng.choice([7, 3, 9], N).astype(np.int32)
    out.append(("msd_cm_both", pos, types, box, "LammpsOrtho", False,
                dict(skip=2, tmax=0, nthreads=3, cm_msd=True, cm_self=True), 9, 1))
    # 3. wrapped positions: the reference wraps the internal copy but takes the
    #    centres of mass from the caller's (unwrapped) positions
    pos = walk(rng, N, T, L, 0.6)
    types = rng.choice([0, 1], N).astype(np.int32)
    out.append(("msd_wrap_cm", pos, types, box, "LammpsOrtho", True,
                dict(skip=1, tmax=5, nthreads=1, cm_msd=True, cm_self=False), 15, 0))
    # 4. non-diagonal cell vectors: the internal positions are rotated, the
    #    centres of mass are not (calc_cm_pos_vel reads the caller's input)
    N, T = 30, 20
    pos = walk(rng, N, T, 6.0, 0.3)
    types = rng.choice([0, 1], N).astype(np.int32)
    cell = np.array([[6.0, 1.0, 0.5], [0.0, 6.0, 0.8], [0.0, 0.0, 6.0]])
    box = np.tile(cell, (T, 1, 1))
    out.append(("msd_rotated_cm_self", pos, types, box, "CellVectors", False,
                dict(skip=2, tmax=4, nthreads=2, cm_msd=False, cm_self=True), 10, 3))
    # 5. a single type, long lags
    N, T, L = 24, 40, 5.0
    pos = walk(rng, N, T, L, 0.2)
    types = np.zeros(N, dtype=np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L], (T, 1))
    out.append(("msd_one_type", pos, types, box, "LammpsOrtho", False,
                dict(skip=5, tmax=20, nthreads=4, cm_msd=True, cm_self=False), 20, 0))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ANALISI_REF"),
                    required="ANALISI_REF" not in os.environ,
                    help="root of the reference tree (or set ANALISI_REF)")
    args = ap.parse_args()
    pa = load_ref(args.ref)
    outdir = os.path.join(HERE, "msd")
    os.makedirs(outdir, exist_ok=True)
    for name, pos, types, box, fmt, wrap, g, n, primo in cases():
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.zeros_like(pos)
        box = np.ascontiguousarray(box, dtype=np.float64)
        tr = pa.Trajectory(pos, vel, types, box, getattr(pa.BoxFormat, fmt), wrap, False)
        m = pa.MeanSquareDisplacement(tr, g["skip"], g["tmax"], g["nthreads"], g["cm_msd"],
                                      g["cm_self"], False)
        m.reset(n)
        m.calculate(primo)
        buf = np.array(m, copy=True)
        meta = dict(g, name=name, box_format=fmt, wrap=wrap, ntimesteps=n, primo=primo,
                    ntypes=int(tr.get_ntypes()))
        np.savez_compressed(
            os.path.join(outdir, name + ".npz"), positions=pos, types=types, box=box,
            ref_buffer=buf, internal_positions=tr.internal_positions().copy(),
            internal_type_ids=tr.internal_type_ids().copy(),
            internal_centres=tr.internal_centres().copy(), meta=json.dumps(meta))
        print(f"{name}: buffer {buf.shape}, sum {buf.sum():.6g}")


if __name__ == "__main__":
    main()
