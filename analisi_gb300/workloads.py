"""Seeded synthetic random-walk trajectories for the five Gofrt workloads.

No public dataset is involved: every workload is a Gaussian random walk of
atoms in a periodic box, generated in FP64 from a fixed seed so that the GPU
engine, the oracle and the reference see identical inputs.

Each generator returns a dict with
  positions  [T][N][3] float64 (raw input, as a user would pass to Trajectory)
  types      [N] int32 raw type labels
  box_lammps [T][6] or [T][9] float64, LAMMPS {xlo,xhi,ylo,yhi,zlo,zhi[,xy,xz,yz]}
  boxes      the same boxes in the reference's internal format
             {xlo,ylo,zlo,lx/2,ly/2,lz/2[,xy,xz,yz]} (lib/include/basetrajectory.h:94-105)
  type_ids   [N] dense ids 0..ntypes-1 in sorted order of the raw labels
             (lib/src/basetrajectory.cpp:52-89)
  ntypes, triclinic, params (the Gofrt arguments of the workload)
With wrap=False and a LAMMPS box the reference uses the positions as they are,
so `positions` are also the internal positions of those workloads.
"""
import math

import numpy as np


def lammps_to_internal(box_lammps):
    """Vectorised restatement of lib/include/basetrajectory.h:94-105."""
    b = np.array(box_lammps, dtype=np.float64, copy=True)
    out = b.copy()
    out[:, 0] = b[:, 0]
    out[:, 1] = b[:, 2]
    out[:, 2] = b[:, 4]
    out[:, 3] = (b[:, 1] - b[:, 0]) / 2
    out[:, 4] = (b[:, 3] - b[:, 2]) / 2
    out[:, 5] = (b[:, 5] - b[:, 4]) / 2
    return out


def dense_type_ids(types):
    """Dense ids in the order of the raw labels compared as unsigned integers
    (lib/src/basetrajectory.cpp:60-79 sorts a std::vector<unsigned int>)."""
    t = np.asarray(types).astype(np.int64) & 0xFFFFFFFF
    u = np.unique(t)
    return np.searchsorted(u, t).astype(np.int32), len(u)


def random_walk(seed, N, T, L, sigma, counts, triclinic_tilt=None, wrap_into_cell=False,
                dtype_chunk=256):
    """Gaussian random walk: frame 0 uniform in the cell, then cumulative
    N(0, sigma^2) steps per axis.  counts: atoms per type (shuffled over atoms)."""
    rng = np.random.default_rng(seed)
    types = np.repeat(np.arange(len(counts), dtype=np.int32), counts)
    rng.shuffle(types)
    pos = np.empty((T, N, 3), dtype=np.float64)
    frac0 = rng.uniform(0.0, 1.0, size=(N, 3))
    if triclinic_tilt is None:
        h = np.diag([L, L, L])
    else:
        xy, xz, yz = triclinic_tilt
        # columns are the cell vectors a=(L,0,0), b=(xy,L,0), c=(xz,yz,L)
        h = np.array([[L, xy, xz], [0.0, L, yz], [0.0, 0.0, L]])
    pos[0] = frac0 @ h.T
    hinv = np.linalg.inv(h)
    # cumulative walk, generated in chunks of frames to bound temporaries
    cur = pos[0].copy()
    for f0 in range(1, T, dtype_chunk):
        f1 = min(T, f0 + dtype_chunk)
        steps = rng.normal(0.0, sigma, size=(f1 - f0, N, 3))
        steps[0] += cur
        np.cumsum(steps, axis=0, out=pos[f0:f1])
        cur = pos[f1 - 1].copy()
    if wrap_into_cell:
        for f in range(T):
            fr = pos[f] @ hinv.T
            fr -= np.floor(fr)
            pos[f] = fr @ h.T
    if triclinic_tilt is None:
        row = np.array([0.0, L, 0.0, L, 0.0, L])
    else:
        row = np.array([0.0, L, 0.0, L, 0.0, L, xy, xz, yz])
    box_lammps = np.tile(row, (T, 1))
    type_ids, ntypes = dense_type_ids(types)
    return {
        "positions": pos, "types": types, "box_lammps": box_lammps,
        "boxes": lammps_to_internal(box_lammps), "type_ids": type_ids, "ntypes": ntypes,
        "triclinic": triclinic_tilt is not None,
    }


def _density_L(N, rho=0.1):
    return (N / rho) ** (1.0 / 3.0)


def c1():
    """Plain FP64 small: N=1000 (500/500), L=22, T=200, sigma=0.05,
    200 bins on [0.7, 3.5], tmax=20, skip=10, reset(180)."""
    w = random_walk(1001, 1000, 200, 22.0, 0.05, [500, 500])
    w["params"] = dict(rmin=0.7, rmax=3.5, nbin=200, tmax=20, skip=10, every=1,
                       ntimesteps=180, primo=0)
    w["name"] = "c1_n1000_fp64_small"
    return w


def c2(T=2000):
    """16k atoms (16352/16/16), density 0.1 (L~54.7), sigma=0.08, T=2000,
    400 bins on [0, 12], lags 0..199, origin stride 4, reset(1800)."""
    N = 16384
    w = random_walk(1002, N, T, _density_L(N), 0.08, [16352, 16, 16])
    w["params"] = dict(rmin=0.0, rmax=12.0, nbin=400, tmax=200, skip=4, every=1,
                       ntimesteps=T - 200, primo=0)
    w["name"] = "c2_n16384_t2000_ortho"
    return w


def c3(T=1000):
    """Triclinic: N=32768 (50/50), cell a=(L,0,0), b=(0.3L,L,0), c=(0.2L,0.1L,L),
    L=70, wrapped into the cell, sigma=0.1, T=1000, 500 bins on [0, 15],
    lags 0..99, origin stride 5, reset(900)."""
    N, L = 32768, 70.0
    w = random_walk(1003, N, T, L, 0.1, [N // 2, N // 2],
                    triclinic_tilt=(0.3 * L, 0.2 * L, 0.1 * L), wrap_into_cell=True)
    w["params"] = dict(rmin=0.0, rmax=15.0, nbin=500, tmax=100, skip=5, every=1,
                       ntimesteps=T - 100, primo=0)
    w["name"] = "c3_n32768_t1000_triclinic"
    return w


def c5(T=500):
    """Large N: N=131072 (4 x 25%), density 0.1 (L~109.5), sigma=0.1, T=500,
    250 bins on [0, 10], lags 0..49, origin stride 10, reset(450)."""
    N = 131072
    w = random_walk(1005, N, T, _density_L(N), 0.1, [N // 4] * 4)
    w["params"] = dict(rmin=0.0, rmax=10.0, nbin=250, tmax=50, skip=10, every=1,
                       ntimesteps=T - 50, primo=0)
    w["name"] = "c5_n131072_t500_cells"
    return w


def c4_member(k):
    """Trajectory k of the 64-trajectory uneven batch (seed 2000+k)."""
    rng = np.random.default_rng(2000 + k)
    N = int(round(math.exp(rng.uniform(math.log(256), math.log(16384)))))
    T = int(rng.integers(100, 1001))
    nt = int(rng.integers(1, 5))
    frac = rng.dirichlet(np.ones(nt))
    counts = np.maximum(1, np.floor(frac * N).astype(int))
    counts[0] += N - counts.sum()
    if counts[0] < 1:  # keep every type populated
        counts = np.ones(nt, dtype=int)
        counts[0] = N - (nt - 1)
    sigma = float(rng.uniform(0.02, 0.15))
    w = random_walk(int(rng.integers(1 << 30)), N, T, _density_L(N), sigma, list(counts))
    tmax = min(100, T // 2)
    n = ((T + 1 - tmax) // 5) * 5
    w["params"] = dict(rmin=0.0, rmax=10.0, nbin=300, tmax=tmax, skip=5, every=1,
                       ntimesteps=n, primo=0)
    w["name"] = f"c4_member{k}_n{N}_t{T}"
    return w


def c4(n=64):
    return [c4_member(k) for k in range(n)]


def pairs_of(N, params):
    """Ordered pairs of the reference loop: N^2 per (lag on the every grid, origin)."""
    p = params
    tmax, n = p["tmax"], p["ntimesteps"]
    leff = n if (n < tmax or tmax == 0) else tmax
    every = p.get("every", 1) or 1
    skip = p.get("skip", 1) or 1
    return ((leff + every - 1) // every) * ((n + skip - 1) // skip) * N * N


def small_case(seed, N, T, L, sigma, counts, tric=False, wrap_into_cell=False, **params):
    tilt = (0.3 * L, 0.2 * L, 0.1 * L) if tric else None
    w = random_walk(seed, N, T, L, sigma, counts, triclinic_tilt=tilt,
                    wrap_into_cell=wrap_into_cell)
    w["params"] = params
    return w
