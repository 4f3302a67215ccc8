"""ctypes front of the C restatement in oracle/gofr_oracle.c -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, always as the checker (or the timed CPU baseline), never as a product
path.  build() compiles the C file with -ffp-contract=off so that the FP64
arithmetic matches the reference's separate multiply/add
(lib/include/basetrajectory.h:215-217) on every host, x86-64 or aarch64.
"""
import ctypes
import os
import subprocess
import sysconfig

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgofr_oracle.so")
SRC = os.path.join(HERE, "gofr_oracle.c")

_lib = None


def build(force=False):
    """Compile oracle/gofr_oracle.c into oracle/_build/libgofr_oracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)):
        return LIB_PATH
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", SRC, "-o", LIB_PATH + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        up = ctypes.POINTER(ctypes.c_uint64)
        L.oracle_d2.argtypes = [dp, dp, dp, ctypes.c_int]
        L.oracle_d2.restype = ctypes.c_double
        L.oracle_bin.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint]
        L.oracle_bin.restype = ctypes.c_int
        L.oracle_channel.argtypes = [ctypes.c_uint] * 3
        L.oracle_channel.restype = ctypes.c_uint
        L.oracle_lammps_to_internal.argtypes = [dp]
        L.oracle_lammps_to_internal.restype = None
        L.oracle_pbc_wrap.argtypes = [dp, dp, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t,
                                      ctypes.c_size_t]
        L.oracle_pbc_wrap.restype = None
        L.oracle_gofrt_counts.argtypes = [dp, dp, ctypes.c_size_t, ctypes.c_int, ip, ctypes.c_uint,
                                          ctypes.c_size_t, ctypes.c_size_t, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_uint, ctypes.c_uint,
                                          ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                          ctypes.c_uint, ctypes.c_size_t, up]
        L.oracle_gofrt_counts.restype = ctypes.c_int
        L.oracle_incr.argtypes = [ctypes.c_uint, ctypes.c_uint]
        L.oracle_incr.restype = ctypes.c_double
        L.oracle_fold_buffer.argtypes = [up, ctypes.c_size_t, ctypes.c_uint, ctypes.c_double, dp]
        L.oracle_fold_buffer.restype = None
        L.oracle_centres.argtypes = [dp, ip, ctypes.c_uint, ctypes.c_size_t, ctypes.c_size_t, dp]
        L.oracle_centres.restype = None
        L.oracle_msd.argtypes = [dp, dp, ip, ctypes.c_uint, ctypes.c_size_t, ctypes.c_size_t,
                                 ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_size_t,
                                 ctypes.c_int, ctypes.c_int, dp]
        L.oracle_msd.restype = ctypes.c_int
        u64p = ctypes.POINTER(ctypes.c_uint64)
        L.oracle_neigh.argtypes = [dp, dp, ctypes.c_size_t, ctypes.c_int, ip, ctypes.c_uint,
                                   ctypes.c_size_t, ctypes.c_size_t, u64p, dp, ctypes.c_int, u64p,
                                   dp, u64p]
        L.oracle_neigh.restype = ctypes.c_int
        L.oracle_sann_n.argtypes = [dp, ctypes.c_uint64]
        L.oracle_sann_n.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def d2(xi, xj, box, tric):
    xi = np.ascontiguousarray(xi, dtype=np.float64)
    xj = np.ascontiguousarray(xj, dtype=np.float64)
    b = np.zeros(9)
    b[:len(box)] = box
    return lib().oracle_d2(_dp(xi), _dp(xj), _dp(b), int(bool(tric)))


def bin_of(d2v, rmin, rmax, nbin):
    return lib().oracle_bin(float(d2v), float(rmin), float(rmax), int(nbin))


def lammps_to_internal(box_rows):
    """Row-wise copy of lib/include/basetrajectory.h:94-105."""
    b = np.array(box_rows, dtype=np.float64, copy=True, order="C")
    for r in range(b.shape[0]):
        lib().oracle_lammps_to_internal(_dp(b[r]))
    return b


def pbc_wrap(pos, boxes, tric):
    """Returns a wrapped copy of pos [T][N][3] (basetrajectory.h:145-161)."""
    p = np.array(pos, dtype=np.float64, copy=True, order="C")
    bx = np.ascontiguousarray(boxes, dtype=np.float64)
    T, N = p.shape[0], p.shape[1]
    for f in range(T):
        lib().oracle_pbc_wrap(_dp(p), _dp(bx), bx.shape[1], int(bool(tric)), N, f)
    return p


def gofrt_counts(pos, boxes, type_ids, ntypes, rmin, rmax, nbin, tmax, nthreads, skip, every,
                 ntimesteps, primo, tric=None, per_thread=False):
    """Integer counts [leff][nch][nbin] (summed over thread partitions unless
    per_thread) of the reference Gofrt on internal buffers."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    boxes = np.ascontiguousarray(boxes, dtype=np.float64)
    type_ids = np.ascontiguousarray(type_ids, dtype=np.int32)
    T, N = pos.shape[0], pos.shape[1]
    stride = boxes.shape[1]
    if tric is None:
        tric = stride == 9
    nthreads = max(1, int(nthreads))
    leff = ntimesteps if (ntimesteps < tmax or tmax == 0) else tmax
    nch = ntypes * (ntypes + 1)
    out = np.zeros((nthreads, leff, nch, nbin), dtype=np.uint64)
    rc = lib().oracle_gofrt_counts(
        _dp(pos), _dp(boxes), stride, int(bool(tric)),
        type_ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ntypes, N, T,
        float(rmin), float(rmax), int(nbin), int(tmax), nthreads, int(skip), int(every),
        int(ntimesteps), int(primo), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    if rc == -1:
        raise RuntimeError("trajectory is too short for this kind of calculation. Select a "
                           "different starting timestep or lower the size of the average or "
                           "the lenght of the time lag")
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return out if per_thread else out.sum(axis=0)


def centres(pos, type_ids, ntypes):
    """Per-frame per-type centres of mass [T][ntypes][3] (running mean over the
    atoms of each type, as the reference's calc_cm_pos_vel)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    type_ids = np.ascontiguousarray(type_ids, dtype=np.int32)
    T, N = pos.shape[0], pos.shape[1]
    cm = np.zeros((T, ntypes, 3))
    lib().oracle_centres(_dp(pos), type_ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                         int(ntypes), N, T, _dp(cm))
    return cm


def msd(pos, type_ids, ntypes, skip, tmax, ntimesteps, primo, cm_msd=False, cm_self=False,
        cm=None):
    """The reference MSD::calculate result [leff][f_cm][ntypes] (running means)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    type_ids = np.ascontiguousarray(type_ids, dtype=np.int32)
    T, N = pos.shape[0], pos.shape[1]
    if cm is None:
        cm = centres(pos, type_ids, ntypes)
    cm = np.ascontiguousarray(cm, dtype=np.float64)
    leff = ntimesteps if (ntimesteps < tmax or tmax == 0) else tmax
    fcm = 2 if cm_msd else 1
    out = np.zeros((leff, fcm, ntypes))
    rc = lib().oracle_msd(_dp(pos), _dp(cm), type_ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                          int(ntypes), N, T, int(skip), int(tmax), int(ntimesteps), int(primo),
                          int(bool(cm_msd)), int(bool(cm_self)), _dp(out))
    if rc == -1:
        raise RuntimeError("trajectory is too short for this kind of calculation. Select a "
                           "different starting timestep or lower the size of the average or "
                           "the lenght of the time lag")
    return out


class NeighLists:
    """The reference's neighbour-list arrays (neighbour.h:68-96) and accessors."""

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
        r = np.ascontiguousarray(self.r(a, k))
        return int(lib().oracle_sann_n(_dp(r), r.shape[0])) if r.size else 0


class TooManyNeighbours(RuntimeError):
    pass


def neighbours(pos, boxes, type_ids, ntypes, timestep, spec, sort):
    """Neighbours(t, spec).update_neigh(timestep, sort) of the reference;
    spec = [(nneigh, cut2, skin2)] per type.  Raises TooManyNeighbours with the
    reference's message."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    boxes = np.ascontiguousarray(boxes, dtype=np.float64)
    type_ids = np.ascontiguousarray(type_ids, dtype=np.int32)
    T, N = pos.shape[0], pos.shape[1]
    nn = np.array([int(s[0]) for s in spec], dtype=np.uint64)
    c2 = np.array([float(s[1]) for s in spec], dtype=np.float64)
    tot = int(nn.sum())
    lst = np.zeros(N * (tot + ntypes), dtype=np.uint64)
    rpos = np.zeros(N * 4 * tot, dtype=np.float64)
    err = np.zeros(6, dtype=np.uint64)
    u64 = ctypes.POINTER(ctypes.c_uint64)
    rc = lib().oracle_neigh(_dp(pos), _dp(boxes), boxes.shape[1], int(boxes.shape[1] == 9),
                            type_ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), int(ntypes), N,
                            int(timestep), nn.ctypes.data_as(u64), _dp(c2), int(bool(sort)),
                            lst.ctypes.data_as(u64), _dp(rpos), err.ctypes.data_as(u64))
    if rc == -1:
        i, j, ni, nj, it, jt = (int(v) for v in err)
        raise TooManyNeighbours(f"Too many neighbours in shell! (iatom={i} jatom={j} ni={ni} "
                                f"nj={nj} itype={it} jtype={jt})")
    return NeighLists(lst, rpos, nn, N)


def incr(ntimesteps, skip):
    return lib().oracle_incr(int(ntimesteps), int(skip))


def fold_buffer(per_thread_counts, incr_value):
    c = np.ascontiguousarray(per_thread_counts, dtype=np.uint64)
    nth = c.shape[0]
    dl = int(np.prod(c.shape[1:]))
    out = np.zeros(c.shape[1:], dtype=np.float64)
    lib().oracle_fold_buffer(c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), dl, nth,
                             float(incr_value), _dp(out))
    return out


def host_info():
    """CPU model and core count of this host (for the CPU-baseline record)."""
    model = "unknown"
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                low = line.lower()
                if low.startswith("model name") or low.startswith("cpu part"):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    return {"cpu": model, "cores": os.cpu_count(), "arch": sysconfig.get_platform()}
