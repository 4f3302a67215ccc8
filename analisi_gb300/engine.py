"""ctypes binding of the C ABI in include/gofr_gb300.h.

This is the thinnest possible host front: it loads the in-tree
libgofr_gb300.so (built by analisi_gb300.build) and fails loudly when it is
missing -- there is no CPU path behind it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgofr_gb300.so")

GOFR_OK = 0
STATUS = {
    -1: "GOFR_ERR_ARG", -2: "GOFR_ERR_RANGE", -3: "GOFR_ERR_CUDA", -4: "GOFR_ERR_NOMEM",
    -5: "GOFR_ERR_STATE", -6: "GOFR_ERR_DEVICE", -7: "GOFR_ERR_UNSUPPORTED",
    -8: "GOFR_ERR_NEIGH_FULL",
}
BOX_ORTHO, BOX_TRICLINIC = 0, 1
KERNELS = {"auto": 0, "f32": 1, "f64": 2, "cell": 3, "tuned": 4, "cellw": 5}

# every symbol the header declares (checked by the CPU tests)
EXPORTED = [
    "gofr_ctx_create", "gofr_ctx_destroy", "gofr_last_error", "gofr_set_frames",
    "gofr_output_size", "gofr_run", "gofr_run_device", "gofr_sync", "gofr_get_stats",
    "gofr_counts_to_buffer", "gofr_bin_thresholds", "gofr_batch_set",
    "gofr_batch_output_layout", "gofr_batch_run", "gofr_measure_peaks",
    "gofr_run_f64_noalloc", "gofr_run_windows", "gofr_set_centres", "gofr_msd_output_size",
    "gofr_msd_run", "gofr_neigh_layout", "gofr_neigh_run", "gofr_run_normalized",
    "gofr_run_streamed", "gofr_cellw_tables", "gofr_plan_query",
]


class NeighLists:
    """The reference's neighbour-list arrays (lib/include/neighbour.h:68-96)
    with its accessors: size, indices, {r, x, y, z} rows, SANN count."""

    def __init__(self, lst, rpos, nneigh, natoms):
        self.list, self.rpos, self.nneigh, self.natoms = lst, rpos, list(nneigh), natoms
        self.loff, self.roff = [0], [0]
        for n in self.nneigh:
            self.loff.append(self.loff[-1] + (n + 1) * natoms)
            self.roff.append(self.roff[-1] + n * natoms * 4)

    def size(self, a, k):
        return int(self.list[self.loff[k] + a * (self.nneigh[k] + 1)])

    def idx(self, a, k):
        b = self.loff[k] + a * (self.nneigh[k] + 1)
        return self.list[b + 1:b + 1 + self.size(a, k)].copy()

    def r(self, a, k):
        b = self.roff[k] + a * self.nneigh[k] * 4
        return self.rpos[b:b + 4 * self.size(a, k)].reshape(-1, 4).copy()

    def sann_n(self, a, k):
        """Neighbours::get_sann_n (lib/src/neighbour.cpp:82-97) on the sorted list."""
        r = self.r(a, k)[:, 0]
        n = len(r)
        if n < 3:
            return 0
        m, s = 3, 0.0
        for i in range(3):
            s += r[i]
        while m < n:
            if s <= r[m] * (m - 2):
                break
            s += r[m]
            m += 1
        return m


class GofrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class TrajectoryTooShort(GofrError):
    pass


class Params(ctypes.Structure):
    _fields_ = [("rmin", ctypes.c_double), ("rmax", ctypes.c_double), ("nbin", ctypes.c_uint),
                ("tmax", ctypes.c_uint), ("skip", ctypes.c_uint), ("every", ctypes.c_uint),
                ("ntimesteps", ctypes.c_uint), ("primo", ctypes.c_ulonglong),
                ("kernel", ctypes.c_int), ("nparts", ctypes.c_uint)]


class MsdParams(ctypes.Structure):
    _fields_ = [("skip", ctypes.c_uint), ("tmax", ctypes.c_uint), ("ntimesteps", ctypes.c_uint),
                ("primo", ctypes.c_ulonglong), ("center_of_mass", ctypes.c_int),
                ("in_center_of_mass_frame", ctypes.c_int)]


class NeighSpec(ctypes.Structure):
    _fields_ = [("nneigh", ctypes.c_ulonglong), ("cut2", ctypes.c_double),
                ("skin2", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_ulonglong), ("evaluated", ctypes.c_ulonglong),
                ("candidates", ctypes.c_ulonglong), ("rechecks", ctypes.c_ulonglong),
                ("kernel_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("kernel_used", ctypes.c_int), ("wrap_checked", ctypes.c_int),
                ("err_bound_d2", ctypes.c_double), ("launches", ctypes.c_ulonglong),
                ("h2d_bytes", ctypes.c_ulonglong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TrajDesc(ctypes.Structure):
    _fields_ = [("positions", ctypes.POINTER(ctypes.c_double)),
                ("boxes", ctypes.POINTER(ctypes.c_double)), ("box_kind", ctypes.c_int),
                ("type_ids", ctypes.POINTER(ctypes.c_int)), ("ntypes", ctypes.c_uint),
                ("natoms", ctypes.c_size_t), ("nframes", ctypes.c_size_t),
                ("params", Params)]


_lib = None


def load_library(path=None):
    """Load libgofr_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} not built: run `python -m analisi_gb300.build` "
                          "(the GPU engine has no CPU fallback)")
    L = ctypes.CDLL(p)
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    up = ctypes.POINTER(ctypes.c_ulonglong)
    L.gofr_ctx_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int]
    L.gofr_ctx_destroy.argtypes = [vp]
    L.gofr_ctx_destroy.restype = None
    L.gofr_last_error.argtypes = [vp]
    L.gofr_last_error.restype = ctypes.c_char_p
    L.gofr_set_frames.argtypes = [vp, dp, dp, ctypes.c_int, ip, ctypes.c_uint, ctypes.c_size_t,
                                  ctypes.c_size_t]
    L.gofr_output_size.argtypes = [vp, ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_size_t)]
    L.gofr_run.argtypes = [vp, ctypes.POINTER(Params), up]
    L.gofr_run_device.argtypes = [vp, ctypes.POINTER(Params), vp]
    L.gofr_sync.argtypes = [vp]
    L.gofr_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.gofr_counts_to_buffer.argtypes = [up, ctypes.c_size_t, ctypes.c_uint, ctypes.c_uint,
                                        ctypes.c_uint, dp]
    L.gofr_bin_thresholds.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_uint, dp]
    L.gofr_cellw_tables.argtypes = [dp, ctypes.c_int, dp, dp, ctypes.c_double, ip, ip,
                                    ctypes.POINTER(ctypes.c_float), dp]
    L.gofr_plan_query.argtypes = [dp, ctypes.c_int, dp, dp, ctypes.c_size_t, ctypes.c_uint,
                                  ctypes.POINTER(Params), ip]
    L.gofr_batch_set.argtypes = [vp, ctypes.POINTER(TrajDesc), ctypes.c_uint]
    L.gofr_batch_output_layout.argtypes = [vp, ctypes.c_uint, ctypes.POINTER(ctypes.c_size_t),
                                           ctypes.POINTER(ctypes.c_size_t)]
    L.gofr_batch_run.argtypes = [vp, ctypes.c_int, up]
    L.gofr_measure_peaks.argtypes = [ctypes.c_int, dp, dp]
    L.gofr_run_windows.argtypes = [vp, ctypes.POINTER(Params), ctypes.c_uint, up, up]
    L.gofr_run_streamed.argtypes = [vp, dp, dp, ctypes.c_int, ip, ctypes.c_uint, ctypes.c_size_t,
                                    ctypes.c_size_t, ctypes.POINTER(Params), ctypes.c_size_t, up]
    L.gofr_run_normalized.argtypes = [vp, ctypes.POINTER(Params), ctypes.c_uint, up, ctypes.c_int,
                                    dp, dp]
    L.gofr_set_centres.argtypes = [vp, dp, ctypes.c_size_t, ctypes.c_uint]
    L.gofr_msd_output_size.argtypes = [vp, ctypes.POINTER(MsdParams),
                                       ctypes.POINTER(ctypes.c_size_t)]
    L.gofr_msd_run.argtypes = [vp, ctypes.POINTER(MsdParams), dp]
    L.gofr_neigh_layout.argtypes = [vp, ctypes.POINTER(NeighSpec), ctypes.c_uint,
                                    ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    L.gofr_neigh_run.argtypes = [vp, ctypes.POINTER(NeighSpec), ctypes.c_uint, ctypes.c_size_t,
                                 ctypes.c_int, up, dp]
    L.gofr_run_f64_noalloc.argtypes = [vp, vp, ctypes.c_int, vp, ctypes.c_uint, ctypes.c_size_t,
                                       ctypes.c_size_t, ctypes.POINTER(Params), vp, vp,
                                       ctypes.c_char_p, ctypes.c_size_t]
    for name in ("gofr_ctx_create", "gofr_set_frames", "gofr_output_size", "gofr_run",
                 "gofr_run_device", "gofr_sync", "gofr_get_stats", "gofr_counts_to_buffer",
                 "gofr_bin_thresholds", "gofr_batch_set", "gofr_batch_output_layout",
                 "gofr_batch_run", "gofr_measure_peaks", "gofr_run_f64_noalloc",
                 "gofr_run_windows", "gofr_run_normalized", "gofr_run_streamed",
                 "gofr_cellw_tables", "gofr_plan_query"):
        getattr(L, name).restype = ctypes.c_int
    if path is None:
        _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_params(rmin, rmax, nbin, tmax=0, skip=1, every=1, ntimesteps=0, primo=0,
                kernel="auto", nparts=1):
    return Params(float(rmin), float(rmax), int(nbin), int(tmax), int(skip), int(every),
                  int(ntimesteps), int(primo), KERNELS[kernel] if isinstance(kernel, str)
                  else int(kernel), int(nparts))


def measure_peaks(device=0):
    """(FP32 lane operations/s, shared-memory u32 atomics/s) measured on the GPU."""
    L = load_library()
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = L.gofr_measure_peaks(int(device), ctypes.byref(a), ctypes.byref(b))
    if rc != GOFR_OK:
        raise GofrError(rc, "peak measurement failed")
    return a.value, b.value


def bin_thresholds(rmin, rmax, nbin):
    """Exact d2 thresholds th[0..nbin] of the reference's bin map (host code)."""
    L = load_library()
    th = np.zeros(int(nbin) + 1)
    rc = L.gofr_bin_thresholds(float(rmin), float(rmax), int(nbin), _dp(th))
    if rc != GOFR_OK:
        raise GofrError(rc, "bin map not monotone for these parameters")
    return th


def plan_query(box, triclinic, coord_min, coord_max, natoms, ntypes, params):
    """The planner's choice for frames in one box (host code, no GPU, tuner
    cache not consulted): a dict {kernel, reach, cells, block, cta_warps,
    wrapcheck}; raises GofrError with gofr_run's status when it would fail."""
    L = load_library()
    b = np.ascontiguousarray(box, dtype=np.float64)
    lo = np.ascontiguousarray(coord_min, dtype=np.float64)
    hi = np.ascontiguousarray(coord_max, dtype=np.float64)
    out = np.zeros(10, dtype=np.int32)
    rc = L.gofr_plan_query(_dp(b), BOX_TRICLINIC if triclinic else BOX_ORTHO, _dp(lo), _dp(hi),
                           int(natoms), int(ntypes), ctypes.byref(params),
                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if rc != GOFR_OK:
        raise GofrError(rc, "the planner refuses these parameters")
    return {"kernel": int(out[0]), "reach": int(out[1]), "cells": tuple(int(v) for v in out[2:5]),
            "block": tuple(int(v) for v in out[5:8]), "cta_warps": int(out[8]),
            "wrapcheck": bool(out[9])}


def cellw_tables(box, triclinic, coord_min, coord_max, rmax, nc):
    """Neighbourhood tables of the warp-streamed cell-list kernel for one box
    (internal format), coordinate extent, rmax and grid (host code): a dict of
    layer, row and cell ranges relative to a warp block, per lattice image,
    the FP32 image vectors [75][3] and the certified per-axis component error
    of the kernel's FP32 differences; None when the kernel refuses the box."""
    L = load_library()
    b = np.ascontiguousarray(box, dtype=np.float64)
    lo = np.ascontiguousarray(coord_min, dtype=np.float64)
    hi = np.ascontiguousarray(coord_max, dtype=np.float64)
    n = np.ascontiguousarray(nc, dtype=np.int32)
    t = np.zeros(38, dtype=np.int32)
    sh = np.zeros((75, 3), dtype=np.float32)
    e = np.zeros(3)
    rc = L.gofr_cellw_tables(_dp(b), BOX_TRICLINIC if triclinic else BOX_ORTHO, _dp(lo), _dp(hi),
                             float(rmax), n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                             t.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                             sh.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), _dp(e))
    if rc == -7:  # GOFR_ERR_UNSUPPORTED
        return None
    if rc != GOFR_OK:
        raise GofrError(rc, "invalid box, extent, rmax or grid")
    return {"nz": (int(t[0]), int(t[1])),
            "ny": {sz: (int(t[2 + sz + 1]), int(t[5 + sz + 1])) for sz in (-1, 0, 1)},
            "nx": {(sz, sy): (int(t[8 + (sz + 1) * 5 + sy + 2]), int(t[23 + (sz + 1) * 5 + sy + 2]))
                   for sz in (-1, 0, 1) for sy in range(-2, 3)},
            "shift": sh, "bound": e}


def counts_to_buffer(counts, ntimesteps, skip, nparts=0):
    """The reference's double result buffer from counts (host code).
    nparts >= 1: counts is [nparts][...] per reference thread partition and the
    result is the reference's exact value (sequential incr sums, folded in
    thread order).  nparts == 0: counts are totals, result counts*incr."""
    L = load_library()
    c = np.ascontiguousarray(counts, dtype=np.uint64)
    shape = c.shape[1:] if nparts >= 1 else c.shape
    n = int(np.prod(shape))
    out = np.zeros(shape, dtype=np.float64)
    rc = L.gofr_counts_to_buffer(c.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)), n,
                                 int(nparts), int(ntimesteps), int(skip), _dp(out))
    if rc != GOFR_OK:
        raise GofrError(rc, "counts_to_buffer failed")
    return out


class Engine:
    """One gofr_ctx: resident frames on one GPU and runs on them."""

    def __init__(self, device=0, library=None):
        """library: a ctypes handle from load_library(path) to use another build
        of the engine (e.g. the GOFR_DEBUG_BOUNDS variant); default the in-tree one."""
        self.L = library if library is not None else load_library()
        self._ctx = ctypes.c_void_p()
        rc = self.L.gofr_ctx_create(ctypes.byref(self._ctx), int(device))
        if rc != GOFR_OK:
            raise GofrError(rc, self.L.gofr_last_error(None).decode())
        self.ntypes = 0
        self.natoms = 0
        self.nframes = 0
        self._batch = None

    def close(self):
        if self._ctx:
            self.L.gofr_ctx_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != GOFR_OK:
            msg = self.L.gofr_last_error(self._ctx).decode()
            cls = TrajectoryTooShort if rc == -2 else GofrError
            raise cls(rc, msg)

    def set_frames(self, positions, boxes, type_ids, ntypes=None, triclinic=None):
        """positions [T][N][3] f64 internal, boxes [T][6|9] f64 internal, type_ids [N]."""
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        bx = np.ascontiguousarray(boxes, dtype=np.float64)
        ty = np.ascontiguousarray(type_ids, dtype=np.int32)
        if triclinic is None:
            triclinic = bx.shape[1] == 9
        if ntypes is None:
            ntypes = int(ty.max()) + 1 if ty.size else 1
        T, N = pos.shape[0], pos.shape[1]
        self._check(self.L.gofr_set_frames(
            self._ctx, _dp(pos), _dp(bx), BOX_TRICLINIC if triclinic else BOX_ORTHO,
            ty.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), int(ntypes), N, T))
        self.ntypes, self.natoms, self.nframes = int(ntypes), N, T

    def set_centres(self, centres):
        """Per-frame per-type centres of mass [T][ntypes][3] (for the MSD
        centre-of-mass options)."""
        cm = np.ascontiguousarray(centres, dtype=np.float64)
        self._check(self.L.gofr_set_centres(self._ctx, _dp(cm), cm.shape[0], cm.shape[1]))

    def msd(self, skip=1, tmax=0, ntimesteps=0, primo=0, center_of_mass=False,
            in_center_of_mass_frame=False):
        """MSD::calculate(primo) after reset(ntimesteps): [leff][f_cm][ntypes] f64."""
        p = MsdParams(int(skip), int(tmax), int(ntimesteps), int(primo), int(bool(center_of_mass)),
                      int(bool(in_center_of_mass_frame)))
        n = ctypes.c_size_t()
        self._check(self.L.gofr_msd_output_size(self._ctx, ctypes.byref(p), ctypes.byref(n)))
        out = np.zeros(max(n.value, 1))
        self._check(self.L.gofr_msd_run(self._ctx, ctypes.byref(p), _dp(out)))
        leff = ntimesteps if (ntimesteps < tmax or tmax == 0) else tmax
        return out[:n.value].reshape(leff, 2 if center_of_mass else 1, self.ntypes)

    def neighbours(self, timestep, spec, sort=True):
        """Neighbours(t, spec).update_neigh(timestep, sort) on the resident
        frames; spec = [(nneigh, cut2, skin2)] per type.  Returns NeighLists."""
        arr = (NeighSpec * len(spec))(*[NeighSpec(int(a), float(b), float(c)) for a, b, c in spec])
        nl, nr = ctypes.c_size_t(), ctypes.c_size_t()
        self._check(self.L.gofr_neigh_layout(self._ctx, arr, len(spec), ctypes.byref(nl),
                                             ctypes.byref(nr)))
        lst = np.zeros(max(nl.value, 1), dtype=np.uint64)
        rpos = np.zeros(max(nr.value, 1))
        self._check(self.L.gofr_neigh_run(
            self._ctx, arr, len(spec), int(timestep), int(bool(sort)),
            lst.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)), _dp(rpos)))
        return NeighLists(lst[:nl.value], rpos[:nr.value], [int(s[0]) for s in spec], self.natoms)

    def output_size(self, params):
        n = ctypes.c_size_t()
        self._check(self.L.gofr_output_size(self._ctx, ctypes.byref(params), ctypes.byref(n)))
        return n.value

    def run(self, rmin, rmax, nbin, tmax=0, skip=1, every=1, ntimesteps=0, primo=0,
            kernel="auto", nparts=1, out=None):
        """Exact counts [leff][nch][nbin] (or [nparts][...]) as uint64."""
        p = make_params(rmin, rmax, nbin, tmax, skip, every, ntimesteps, primo, kernel, nparts)
        n = self.output_size(p)
        leff = ntimesteps if (ntimesteps < tmax or tmax == 0) else tmax
        nch = self.ntypes * (self.ntypes + 1)
        shape = (leff, nch, int(nbin)) if nparts <= 1 else (int(nparts), leff, nch, int(nbin))
        if out is None:
            out = np.zeros(max(n, 1), dtype=np.uint64)
        self._check(self.L.gofr_run(self._ctx, ctypes.byref(p),
                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong))))
        return out[:n].reshape(shape)

    def run_windows(self, rmin, rmax, nbin, tmax, skip, every, ntimesteps, primos,
                    kernel="auto", nparts=1):
        """Counts of several calculate(primo) windows in one launch:
        [nwin][leff][nch][nbin] (or [nwin][nparts][...] when nparts > 1)."""
        primos = np.ascontiguousarray(primos, dtype=np.uint64)
        p = make_params(rmin, rmax, nbin, tmax, skip, every, ntimesteps, 0, kernel, nparts)
        n = self.output_size(p)
        leff = ntimesteps if (ntimesteps < tmax or tmax == 0) else tmax
        nch = self.ntypes * (self.ntypes + 1)
        out = np.zeros(max(n * len(primos), 1), dtype=np.uint64)
        self._check(self.L.gofr_run_windows(
            self._ctx, ctypes.byref(p), len(primos),
            primos.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)),
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong))))
        shape = (len(primos), leff, nch, int(nbin)) if nparts <= 1 else \
            (len(primos), int(nparts), leff, nch, int(nbin))
        return out[:n * len(primos)].reshape(shape)

    def run_streamed(self, positions, boxes, type_ids, ntypes, max_device_bytes, rmin, rmax, nbin,
                     tmax=0, skip=1, every=1, ntimesteps=0, primo=0, kernel="auto", nparts=1):
        """gofr_run on host frames streamed through the device in chunks of
        origins whose frames fit max_device_bytes (the context's resident
        frames are replaced by the last chunk's)."""
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        bx = np.ascontiguousarray(boxes, dtype=np.float64)
        ty = np.ascontiguousarray(type_ids, dtype=np.int32)
        p = make_params(rmin, rmax, nbin, tmax, skip, every, ntimesteps, primo, kernel, nparts)
        leff = ntimesteps if (ntimesteps < tmax or tmax == 0) else tmax
        nch = int(ntypes) * (int(ntypes) + 1)
        shape = (leff, nch, int(nbin)) if nparts <= 1 else (int(nparts), leff, nch, int(nbin))
        out = np.zeros(max(int(np.prod(shape)), 1), dtype=np.uint64)
        self._check(self.L.gofr_run_streamed(
            self._ctx, _dp(pos), _dp(bx), BOX_TRICLINIC if bx.shape[1] == 9 else BOX_ORTHO,
            ty.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), int(ntypes), pos.shape[1],
            pos.shape[0], ctypes.byref(p), int(max_device_bytes),
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong))))
        self.ntypes, self.natoms, self.nframes = int(ntypes), pos.shape[1], pos.shape[0]
        return out[:int(np.prod(shape))].reshape(shape)

    NORMS = {"buffer": 0, "shell": 1, "density": 2}

    def gofr(self, rmin, rmax, nbin, tmax, skip, every, ntimesteps, primos, norm="shell",
             nparts=1, kernel="auto"):
        """calculate(primo) for each primo of `primos` with the result made into
        doubles on the GPU: norm "buffer" (the reference's Gofrt buffer, bit for
        bit), "shell" (divided by the shell volumes: the reference's hist2gofr)
        or "density" (also by each channel's pair density).  Returns
        ([nwin][leff][nch][nbin] float64, bound on the relative difference from
        a host FP64 evaluation of the same formula)."""
        primos = np.ascontiguousarray(np.atleast_1d(primos), dtype=np.uint64)
        p = make_params(rmin, rmax, nbin, tmax, skip, every, ntimesteps, 0, kernel, nparts)
        leff = ntimesteps if (ntimesteps < tmax or tmax == 0) else tmax
        nch = self.ntypes * (self.ntypes + 1)
        out = np.zeros(max(len(primos) * leff * nch * int(nbin), 1))
        bound = ctypes.c_double()
        self._check(self.L.gofr_run_normalized(
            self._ctx, ctypes.byref(p), len(primos),
            primos.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)),
            self.NORMS[norm] if isinstance(norm, str) else int(norm), _dp(out),
            ctypes.byref(bound)))
        return out[:len(primos) * leff * nch * int(nbin)].reshape(
            len(primos), leff, nch, int(nbin)), bound.value

    def run_params(self, p, out):
        """gofr_run with prepared Params and a preallocated uint64 output (hot loop form)."""
        self._check(self.L.gofr_run(self._ctx, ctypes.byref(p),
                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong))))
        return out

    def run_device(self, p, dev_ptr):
        self._check(self.L.gofr_run_device(self._ctx, ctypes.byref(p), ctypes.c_void_p(dev_ptr)))

    def sync(self):
        self._check(self.L.gofr_sync(self._ctx))

    def stats(self):
        s = Stats()
        self._check(self.L.gofr_get_stats(self._ctx, ctypes.byref(s)))
        return s.as_dict()

    # ---- batches ---------------------------------------------------------
    def batch_set(self, trajs):
        """trajs: list of dicts with positions, boxes, type_ids, ntypes, params (Params)."""
        keep = []
        descs = (TrajDesc * len(trajs))()
        for k, t in enumerate(trajs):
            pos = np.ascontiguousarray(t["positions"], dtype=np.float64)
            bx = np.ascontiguousarray(t["boxes"], dtype=np.float64)
            ty = np.ascontiguousarray(t["type_ids"], dtype=np.int32)
            keep += [pos, bx, ty]
            descs[k] = TrajDesc(_dp(pos), _dp(bx),
                                BOX_TRICLINIC if bx.shape[1] == 9 else BOX_ORTHO,
                                ty.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                int(t["ntypes"]), pos.shape[1], pos.shape[0], t["params"])
        self._check(self.L.gofr_batch_set(self._ctx, descs, len(trajs)))
        layout = []
        total = 0
        for k, t in enumerate(trajs):
            off, n = ctypes.c_size_t(), ctypes.c_size_t()
            self._check(self.L.gofr_batch_output_layout(self._ctx, k, ctypes.byref(off),
                                                        ctypes.byref(n)))
            p = t["params"]
            leff = p.ntimesteps if (p.ntimesteps < p.tmax or p.tmax == 0) else p.tmax
            nch = int(t["ntypes"]) * (int(t["ntypes"]) + 1)
            layout.append((off.value, n.value, (leff, nch, p.nbin)))
            total = max(total, off.value + n.value)
        self._batch = (layout, total)
        return layout

    def batch_run(self, use_graph=True, out=None):
        layout, total = self._batch
        if out is None:
            out = np.zeros(max(total, 1), dtype=np.uint64)
        self._check(self.L.gofr_batch_run(self._ctx, int(bool(use_graph)),
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong))))
        return [out[o:o + n].reshape(s) for (o, n, s) in layout]
