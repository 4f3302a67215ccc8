"""Generates tests/golden/*.npz with the reference's own Gofrt build.

Run where the analisi source tree is present (it builds oracle/_ref with
oracle/build_ref.sh if needed):

    python tests/golden/make_golden.py [--ref /path/to/analisi]

Each fixture holds a small seeded input (raw arrays as a user passes them to
pyanalisi.Trajectory), the Gofrt arguments, and what the reference computed:
its result buffer (double, with its own thread fold) and its internal
(post-preprocessing) positions, boxes and type ids.  The reference's own gofr
regression inputs are not available (.MISSING_LARGE_BLOBS), so these seeded
cases stand in for them; they exercise the same API calls as the reference's
tests/test_gofrt.py and tests/src/test_lammps2020.cpp.
"""
import argparse
import glob
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def load_ref(ref_root):
    out = os.path.join(ROOT, "oracle", "_ref")
    if not glob.glob(os.path.join(out, "pyanalisi_ref*.so")):
        subprocess.check_call(["sh", os.path.join(ROOT, "oracle", "build_ref.sh"), ref_root])
    sys.path.insert(0, out)
    import pyanalisi_ref
    return pyanalisi_ref


def walk(rng, N, T, L, sigma, start=None):
    p0 = rng.uniform(0, L, (N, 3)) if start is None else start
    steps = rng.normal(0, sigma, (T - 1, N, 3))
    return np.concatenate([p0[None], p0[None] + np.cumsum(steps, axis=0)])


def cases():
    """(name, raw inputs, box format, wrap, Gofrt args, reset n, primo)."""
    out = []
    rng = np.random.default_rng(20240)
    # 1. orthorhombic LAMMPS box, two raw type labels, 3 threads, primo > 0
    N, T, L = 48, 30, 7.0
    pos = walk(rng, N, T, L, 0.3)
    types = rng.choice([5, 9], N).astype(np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L], (T, 1))
    out.append(("ortho_lammps", pos, types, box, "LammpsOrtho", False,
                dict(rmin=0.0, rmax=3.4, nbin=40, tmax=6, nthreads=3, skip=4, every=1), 20, 2))
    # 2. same box with wrapping, 4 threads, every=2, rmin > 0, skip not dividing n
    pos = walk(rng, N, T, L, 0.4)
    types = rng.choice([1, 2, 3], N).astype(np.int32)
    box = np.tile([-1.0, L - 1.0, 0.5, L + 0.5, 0.0, L * 1.1], (T, 1))
    out.append(("ortho_wrap", pos, types, box, "LammpsOrtho", True,
                dict(rmin=0.5, rmax=3.3, nbin=33, tmax=8, nthreads=4, skip=3, every=2), 17, 1))
    # 3. triclinic LAMMPS box (tilts).  wrap=True: with LammpsTriclinic and
    #    wrap=False the reference allocates its internal positions but never
    #    copies the input into them (lib/src/trajectory_numpy.cpp:185-213), so
    #    that combination computes on uninitialised memory.
    N, T, L = 40, 24, 8.0
    pos = walk(rng, N, T, L, 0.3)
    types = np.zeros(N, dtype=np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L, 0.3 * L, 0.2 * L, 0.1 * L], (T, 1))
    out.append(("tric_lammps", pos, types, box, "LammpsTriclinic", True,
                dict(rmin=0.0, rmax=3.9, nbin=50, tmax=5, nthreads=2, skip=7, every=1), 16, 0))
    # 4. triclinic with wrapping
    pos = walk(rng, N, T, L, 0.5)
    types = rng.choice([0, 1], N).astype(np.int32)
    out.append(("tric_wrap", pos, types, box, "LammpsTriclinic", True,
                dict(rmin=0.2, rmax=3.9, nbin=45, tmax=4, nthreads=3, skip=2, every=1), 18, 2))
    # 5. diagonal cell vectors (no rotation), tmax=0 (leff = n)
    N, T, L = 36, 20, 6.5
    pos = walk(rng, N, T, L, 0.2)
    types = rng.choice([2, 7], N).astype(np.int32)
    cells = np.tile(np.diag([L, L * 1.05, L * 0.95])[None], (T, 1, 1))
    out.append(("cellvec_diag", pos, types, cells, "CellVectors", False,
                dict(rmin=0.0, rmax=3.0, nbin=30, tmax=0, nthreads=1, skip=2, every=1), 9, 1))
    # 6. non-diagonal cell vectors: the reference rotates positions (QR)
    a1, a2, a3 = np.array([L, 0.4, 0.0]), np.array([0.7, L, 0.3]), np.array([0.2, -0.5, L])
    cells = np.tile(np.stack([a1, a2, a3], axis=1)[None], (T, 1, 1))  # columns = cell vectors
    pos = walk(rng, N, T, L, 0.2)
    out.append(("cellvec_tric", pos, types, np.ascontiguousarray(cells), "CellVectors", False,
                dict(rmin=0.0, rmax=3.1, nbin=31, tmax=3, nthreads=2, skip=3, every=1), 12, 0))
    # 7. small box, far unwrapped coordinates (several boxes away): multi-step
    #    minimum image and rmax > l/2
    N, T, L = 30, 16, 4.0
    pos = walk(rng, N, T, L, 0.6) + rng.integers(-3, 4, (1, N, 3)) * L
    types = rng.choice([0, 1], N).astype(np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L], (T, 1))
    out.append(("small_box_far", pos, types, box, "LammpsOrtho", False,
                dict(rmin=0.0, rmax=3.2, nbin=64, tmax=4, nthreads=2, skip=2, every=1), 10, 1))
    # 8. known answers at bin edges: two atoms per frame at chosen distances
    #    d = 0.2999999999 with dr = 0.1 lands in bin 3 (float rounding of the
    #    quotient), d = 0.9999999999 with rmax = 1 is dropped, |dx| == l/2 is
    #    not wrapped.
    L = 10.0
    ds = [0.2999999999, 0.9999999999, 0.45, 0.05, 5.0, 0.1, 0.7000000001]
    T = len(ds)
    pos = np.zeros((T, 2, 3))
    for f, d in enumerate(ds):
        pos[f, 0] = [1.0, 1.0, 1.0]
        pos[f, 1] = [1.0 + d, 1.0, 1.0]
    types = np.array([0, 1], dtype=np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L], (T, 1))
    out.append(("kat_bin_edges", pos, types, box, "LammpsOrtho", False,
                dict(rmin=0.0, rmax=1.0, nbin=10, tmax=1, nthreads=1, skip=1, every=1), T, 0))
    # 9. self channel at lag 0 with rmin = 0: every atom in bin 0
    N, T, L = 25, 10, 5.0
    pos = walk(rng, N, T, L, 0.1)
    types = rng.choice([0, 1, 2], N).astype(np.int32)
    box = np.tile([0.0, L, 0.0, L, 0.0, L], (T, 1))
    out.append(("self_lag0", pos, types, box, "LammpsOrtho", False,
                dict(rmin=0.0, rmax=2.0, nbin=20, tmax=1, nthreads=1, skip=1, every=1), 7, 0))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ANALISI_REF"),
                    required="ANALISI_REF" not in os.environ,
                    help="root of the reference tree (or set ANALISI_REF)")
    args = ap.parse_args()
    pa = load_ref(args.ref)
    for name, pos, types, box, fmt, wrap, g, n, primo in cases():
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.zeros_like(pos)
        box = np.ascontiguousarray(box, dtype=np.float64)
        tr = pa.Trajectory(pos, vel, types, box, getattr(pa.BoxFormat, fmt), wrap, False)
        gofr = pa.Gofrt(tr, g["rmin"], g["rmax"], g["nbin"], g["tmax"], g["nthreads"], g["skip"],
                        g["every"], False)
        gofr.reset(n)
        gofr.calculate(primo)
        buf = np.array(gofr, copy=True)
        meta = dict(g, name=name, box_format=fmt, wrap=wrap, ntimesteps=n, primo=primo,
                    ntypes=int(tr.get_ntypes()), triclinic=bool(tr.is_triclinic()),
                    columns=gofr.get_columns_description())
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), positions=pos, types=types, box=box,
            ref_buffer=buf, internal_positions=tr.internal_positions().copy(),
            internal_boxes=tr.internal_boxes().copy(),
            internal_type_ids=tr.internal_type_ids().copy(), meta=json.dumps(meta))
        print(f"{name}: buffer {buf.shape}, sum {buf.sum():.6g}")


if __name__ == "__main__":
    main()
