"""The certified error bound of the warp-streamed cell-list kernel, checked
numerically on the CPU.

For pairs the reference counts (reference image distance < rmax), the
kernel's FP32 arithmetic is replayed in numpy -- coordinates reduced into the
cell by the lattice in FP64 and rounded to FP32 about the box centre, the
neighbour moved by the FP32 image vector of the host's table, FP32
differences, d2 as a multiply and two FMAs -- and compared with the
reference's own FP64 minimum image and d2 (lib/include/basetrajectory.h:
200-268): every component must lie within the per-axis bound the host
certifies (gofr_cellw_tables, the bound the kernel's windows are built from),
and d2 within the bound's E(d2), for orthorhombic and triclinic boxes,
shifted boxes and coordinates several lattice vectors outside the cell."""
import math

import numpy as np
import pytest

from analisi_gb300 import engine


def ref_image(d, L, tilt):
    """The reference's iterative minimum image, z then y then x, strict '>'."""
    xy, xz, yz = tilt
    d = d.copy()
    for _ in range(64):
        m = d[:, 2] > L[2] / 2
        d[m, 2] -= L[2]; d[m, 1] -= yz; d[m, 0] -= xz
        m = d[:, 2] < -L[2] / 2
        d[m, 2] += L[2]; d[m, 1] += yz; d[m, 0] += xz
    for _ in range(64):
        m = d[:, 1] > L[1] / 2
        d[m, 1] -= L[1]; d[m, 0] -= xy
        m = d[:, 1] < -L[1] / 2
        d[m, 1] += L[1]; d[m, 0] += xy
    for _ in range(64):
        m = d[:, 0] > L[0] / 2
        d[m, 0] -= L[0]
        m = d[:, 0] < -L[0] / 2
        d[m, 0] += L[0]
    return d


def ref_d2(d):
    """((0 + x*x) + y*y) + z*z in FP64, as the reference sums it."""
    return (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]


def reduce_into_cell(p, lo, L, tilt):
    xy, xz, yz = tilt
    w = p.copy()
    nz = np.floor((w[:, 2] - lo[2]) / L[2])
    w[:, 2] -= nz * L[2]; w[:, 1] -= nz * yz; w[:, 0] -= nz * xz
    ny = np.floor((w[:, 1] - lo[1]) / L[1])
    w[:, 1] -= ny * L[1]; w[:, 0] -= ny * xy
    nx = np.floor((w[:, 0] - lo[0]) / L[0])
    w[:, 0] -= nx * L[0]
    return w


def fma32(a, b, c):
    """fl32(a b + c) (a b is exact in FP64 for FP32 a, b)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


BOXES = [
    # L3, tilt {xy, xz, yz}, lo, lattice vectors out, rmax
    ((70.0, 70.0, 70.0), (21.0, 14.0, 7.0), (0.0, 0.0, 0.0), 0, 15.0),
    ((26.0, 31.0, 35.0), (-8.0, 11.0, -13.0), (-3.0, 2.5, 7.0), 3, 6.0),
    ((24.0, 24.0, 24.0), (12.0, -12.0, 12.0), (100.0, -50.0, 20.0), 5, 5.0),
    ((54.72, 54.72, 54.72), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0, 12.0),
    ((27.0, 25.0, 29.0), (0.0, 0.0, 0.0), (4.0, -6.0, 1.5), 40, 5.5),
]


@pytest.mark.parametrize("box", BOXES, ids=[str(i) for i in range(len(BOXES))])
def test_fp32_cell_differences_within_the_certified_bound(built_engine, box):
    L3, tilt, lo, out, rmax = box
    tric = any(t != 0.0 for t in tilt)
    L = np.array(L3)
    lo = np.array(lo)
    H = np.array([[L[0], 0, 0], [tilt[0], L[1], 0], [tilt[1], tilt[2], L[2]]])  # rows a, b, c
    rng = np.random.default_rng(11)
    n = 200000
    xi = rng.random((n, 3)) @ H + lo + rng.integers(-out, out + 1, (n, 3)) @ H
    # partners within rmax of the first atom's image, moved by random lattice vectors
    v = rng.normal(size=(n, 3))
    v *= (rmax * rng.random(n) ** (1 / 3) / np.linalg.norm(v, axis=1))[:, None]
    xj = xi - v + rng.integers(-out - 1, out + 2, (n, 3)) @ H
    d_ref = ref_image(xi - xj, L, tilt if tric else (0.0, 0.0, 0.0))
    s_ref = ref_d2(d_ref)
    keep = s_ref < rmax * rmax
    xi, xj, d_ref, s_ref = xi[keep], xj[keep], d_ref[keep], s_ref[keep]
    allx = np.concatenate([xi, xj])
    internal = list(lo) + list(L / 2) + (list(tilt) if tric else [])
    nc = [max(3, math.floor(L[k] / (rmax * (1 + 1e-6)))) for k in range(3)]
    tab = engine.cellw_tables(internal, tric, allx.min(0), allx.max(0), rmax, nc)
    assert tab is not None
    e = tab["bound"]
    # the kernel's records: reduced into the cell in FP64, FP32 about the centre
    c = lo + L / 2
    wi = reduce_into_cell(xi, lo, L, tilt if tric else (0.0, 0.0, 0.0))
    wj = reduce_into_cell(xj, lo, L, tilt if tric else (0.0, 0.0, 0.0))
    ai = (wi - c).astype(np.float32)
    aj = (wj - c).astype(np.float32)
    # the lattice image the neighbourhood reaches j in, and its FP32 vector from the table
    D = (wi - wj) - d_ref
    sz = np.rint(D[:, 2] / L[2])
    sy = np.rint((D[:, 1] - sz * (tilt[2] if tric else 0.0)) / L[1])
    sx = np.rint((D[:, 0] - sz * (tilt[1] if tric else 0.0) - sy * (tilt[0] if tric else 0.0)) / L[0])
    assert np.all(np.abs(sx) <= 2) and np.all(np.abs(sy) <= 2) and np.all(np.abs(sz) <= 1)
    idx = ((sx + 2) + 5 * (sy + 2) + 25 * (sz + 1)).astype(int)
    sh = tab["shift"][idx]
    b = (aj + sh).astype(np.float32)
    dx = (ai - b).astype(np.float32)
    # components within the certified per-axis bound
    err = np.abs(dx.astype(np.float64) - d_ref)
    assert np.all(err <= e[None, :]), (err.max(0), e)
    # d2 (a multiply, two FMAs) within E(d2)
    d2 = fma32(dx[:, 2], dx[:, 2], fma32(dx[:, 1], dx[:, 1], dx[:, 0] * dx[:, 0]))
    en = float(np.linalg.norm(e))
    E = (2 * np.sqrt(s_ref) * en + 2 * en * en + 5.01 * 2.0 ** -24 * s_ref) * (1 + 2.0 ** -20)
    assert np.all(np.abs(d2.astype(np.float64) - s_ref) <= E)
    # the bound is not vacuous: the observed error reaches a visible share of it
    assert err.max() > 0.01 * e.min()
