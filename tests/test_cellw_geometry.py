"""Neighbourhood geometry of the warp-streamed cell-list kernel, on the CPU.

The kernel's neighbourhood tables (gofr_cellw_tables: the same host code the
GPU path launches with) are walked here exactly as the kernel walks them --
layers, rows per layer image, cells per row image, one or two pieces per row
-- for every warp block of a grid, and the pairs they reach are compared with
a brute-force evaluation of the reference's minimum image (z, then y, then x,
strict '>'; lib/include/basetrajectory.h:224-268): every pair the reference
counts (distance < rmax) must be reached exactly once, in the lattice image
whose difference vector is the reference's.  Orthorhombic, triclinic
(positive, negative and half-box tilts), shifted boxes, atoms several lattice
vectors outside the cell, reach 1 to 3."""
import math

import numpy as np
import pytest

from analisi_gb300 import engine


def ref_image(d, L, tilt):
    """The reference's iterative minimum image of difference vectors d [..., 3]."""
    xy, xz, yz = tilt
    d = d.copy()
    for _ in range(16):
        m = d[..., 2] > L[2] / 2
        d[..., 2][m] -= L[2]; d[..., 1][m] -= yz; d[..., 0][m] -= xz
        m = d[..., 2] < -L[2] / 2
        d[..., 2][m] += L[2]; d[..., 1][m] += yz; d[..., 0][m] += xz
    for _ in range(16):
        m = d[..., 1] > L[1] / 2
        d[..., 1][m] -= L[1]; d[..., 0][m] -= xy
        m = d[..., 1] < -L[1] / 2
        d[..., 1][m] += L[1]; d[..., 0][m] += xy
    for _ in range(16):
        m = d[..., 0] > L[0] / 2
        d[..., 0][m] -= L[0]
        m = d[..., 0] < -L[0] / 2
        d[..., 0][m] += L[0]
    return d


def reduce_into_cell(p, lo, L, tilt, tric):
    """Coordinates moved into [lo, lo + L) by the lattice (z, y, x), as the
    kernel's cell build does, and the atoms' cells on the grid nc."""
    xy, xz, yz = tilt if tric else (0.0, 0.0, 0.0)
    w = p.copy()
    nz = np.floor((w[:, 2] - lo[2]) / L[2])
    w[:, 2] -= nz * L[2]; w[:, 1] -= nz * yz; w[:, 0] -= nz * xz
    ny = np.floor((w[:, 1] - lo[1]) / L[1])
    w[:, 1] -= ny * L[1]; w[:, 0] -= ny * xy
    nx = np.floor((w[:, 0] - lo[0]) / L[0])
    w[:, 0] -= nx * L[0]
    return w


def check_grid(box, tric, pos, rmax, m, wblk):
    lo = np.array(box[:3])
    L = 2.0 * np.array(box[3:6])
    tilt = tuple(box[6:9]) if tric else (0.0, 0.0, 0.0)
    nc = [math.floor(L[k] * m / (rmax * (1 + 1e-6))) for k in range(3)]
    if any(n < 2 * m + 1 for n in nc):
        return None
    tab = engine.cellw_tables(box, tric, pos.min(0), pos.max(0), rmax, nc)
    if tab is None:
        return None
    nz_lo, nz_hi = tab["nz"]
    ny_span = max(hi - lo_ + 1 for lo_, hi in tab["ny"].values())
    nx_span = max(hi - lo_ + 1 for lo_, hi in tab["nx"].values())
    # the planner's conditions on a warp block
    if any(wblk[k] + 2 * m > nc[k] for k in range(3)) or wblk[0] + nx_span > nc[0]:
        return None
    if (wblk[1] + ny_span) * (wblk[2] + nz_hi - nz_lo + 1) > 64:
        return None
    w = reduce_into_cell(pos, lo, L, tilt, tric)
    cell = np.clip(np.floor((w - lo) / L * np.array(nc)).astype(int), 0, np.array(nc) - 1)
    cid = (cell[:, 2] * nc[1] + cell[:, 1]) * nc[0] + cell[:, 0]
    members = [np.nonzero(cid == c)[0] for c in range(nc[0] * nc[1] * nc[2])]
    H = np.array([[L[0], 0, 0], [tilt[0], L[1], 0], [tilt[1], tilt[2], L[2]]])  # rows a, b, c
    N = pos.shape[0]
    d_ref = ref_image(pos[:, None, :] - pos[None, :, :], L, tilt)
    want = (d_ref ** 2).sum(-1) < rmax * rmax
    got = np.zeros((N, N), dtype=int)
    nw = [(nc[k] + wblk[k] - 1) // wblk[k] for k in range(3)]
    for wz in range(nw[2]):
        for wy in range(nw[1]):
            for wx in range(nw[0]):
                c0 = [wx * wblk[0], wy * wblk[1], wz * wblk[2]]
                cn = [min(wblk[k], nc[k] - c0[k]) for k in range(3)]
                first = np.concatenate([members[(cz * nc[1] + cy) * nc[0] + cx]
                                        for cz in range(c0[2], c0[2] + cn[2])
                                        for cy in range(c0[1], c0[1] + cn[1])
                                        for cx in range(c0[0], c0[0] + cn[0])])
                if first.size == 0:
                    continue
                js, shifts = [], []
                jny = cn[1] + ny_span
                for rr in range((cn[2] + nz_hi - nz_lo + 1) * jny):
                    lz, k = divmod(rr, jny)
                    uz = c0[2] + nz_lo + lz
                    sz, cz = divmod(uz, nc[2])
                    ylo, yhi = tab["ny"][sz]
                    if k > cn[1] + yhi - ylo:
                        continue
                    uy = c0[1] + ylo + k
                    sy, cy = divmod(uy, nc[1])
                    xlo, xhi = tab["nx"][(sz, sy)]
                    for ux in range(c0[0] + xlo, c0[0] + cn[0] + xhi + 1):
                        sx, cx = divmod(ux, nc[0])
                        mem = members[(cz * nc[1] + cy) * nc[0] + cx]
                        js.append(mem)
                        shifts.append(np.repeat((sx * H[0] + sy * H[1] + sz * H[2])[None],
                                                mem.size, 0))
                js = np.concatenate(js)
                shifts = np.concatenate(shifts)
                d = w[first][:, None, :] - (w[js] + shifts)[None, :, :]
                inr = (d ** 2).sum(-1) < rmax * rmax
                for a, i in enumerate(first):
                    for b in np.nonzero(inr[a])[0]:
                        got[i, js[b]] += 1
                        np.testing.assert_allclose(d[a, b], d_ref[i, js[b]], atol=1e-9)
    assert np.array_equal(got, want.astype(int))
    return int(want.sum())


def lattice_case(seed, N, L3, tilt, lo, unwrap):
    rng = np.random.default_rng(seed)
    H = np.array([[L3[0], 0, 0], [tilt[0], L3[1], 0], [tilt[1], tilt[2], L3[2]]])
    f = rng.random((N, 3)) + rng.integers(-unwrap, unwrap + 1, (N, 3))
    return f @ H + np.array(lo)


BOXES = [
    # L3, tilt {xy, xz, yz}, lo, unwrap, rmax
    ((30.0, 30.0, 30.0), (9.0, 6.0, 3.0), (0.0, 0.0, 0.0), 0, 7.0),
    ((26.0, 31.0, 35.0), (-8.0, 11.0, -13.0), (-3.0, 2.5, 7.0), 2, 6.0),
    ((24.0, 24.0, 24.0), (12.0, -12.0, 12.0), (0.0, 0.0, 0.0), 1, 5.0),
    ((27.0, 25.0, 29.0), (0.0, 0.0, 0.0), (4.0, -6.0, 1.5), 2, 5.5),
]


@pytest.mark.parametrize("m,wblk", [(1, (1, 1, 1)), (2, (1, 1, 1)), (2, (2, 1, 2)), (3, (1, 1, 1)),
                                    (3, (2, 2, 1))])
@pytest.mark.parametrize("box", BOXES, ids=[str(i) for i in range(len(BOXES))])
def test_every_counted_pair_is_reached_once_in_its_reference_image(built_engine, box, m, wblk):
    L3, tilt, lo, unwrap, rmax = box
    pos = lattice_case(7 + m, 700, L3, tilt, lo, unwrap)
    tric = any(t != 0.0 for t in tilt)
    internal = [lo[0], lo[1], lo[2], L3[0] / 2, L3[1] / 2, L3[2] / 2] + \
        (list(tilt) if tric else [])
    n = check_grid(internal, tric, pos, rmax, m, wblk)
    if n is None:
        pytest.skip("no grid or warp block of this shape for this box")
    assert n > 0


def test_orthorhombic_tables_are_the_whole_cell_reach(built_engine):
    """Orthorhombic grids reach exactly -reach .. reach-1 cells beyond the
    block on every axis, every image in -1..1 with vector s fl32(L)."""
    for m in (1, 2, 3):
        L = 40.0
        nc = [math.floor(L * m / (6.0 * (1 + 1e-6)))] * 3
        tab = engine.cellw_tables([1.0, -2.0, 0.5, L / 2, L / 2, L / 2], False, [1.0, -2.0, 0.5],
                                  [41.0, 38.0, 40.5], 6.0, nc)
        assert tab["nz"] == (-m, m - 1)
        assert all(tab["ny"][sz] == (-m, m - 1) for sz in (-1, 0, 1))
        assert all(tab["nx"][(sz, sy)] == (-m, m - 1) for sz in (-1, 0, 1) for sy in (-1, 0, 1))
        for sx in (-1, 0, 1):
            for sy in (-1, 0, 1):
                for sz in (-1, 0, 1):
                    v = tab["shift"][(sx + 2) + 5 * (sy + 2) + 25 * (sz + 1)]
                    assert tuple(v) == (np.float32(sx * L), np.float32(sy * L),
                                        np.float32(sz * L))


def test_tilts_beyond_the_image_table_are_refused(built_engine):
    """xy = 2.7 Lx reaches x images three box lengths away: no tables (the
    kernel refuses the box and the planner takes the all-pairs kernel)."""
    assert engine.cellw_tables([0, 0, 0, 10, 10, 10, 54, 0, 0], True, [0, 0, 0], [20, 20, 20],
                               4.0, [7, 7, 7]) is None
    with pytest.raises(engine.GofrError):
        engine.cellw_tables([0, 0, 0, -1, 10, 10], False, [0, 0, 0], [20, 20, 20], 4.0, [7, 7, 7])
