"""The reference's Python g(r) conveniences on the GB300 engine.

Restates pyanalisi/analysis.py:77-86 (max_l), :101-105 (hist2gofr) and
:108-145 (Analysis.compute_gofr) -- equivalently pyanalisi/common.py:186-206
(analyze_gofr) -- for a trajectory of this package's `pyanalisi` module.
The segmented form (n_segments > 1), a loop of Gofrt::calculate calls in the
reference, runs every segment of the resident frames in one persistent
launch (gofr_run_normalized).  The histograms are the reference's exact
doubles: the counts of each reference thread partition are folded as its
threads add incr, on the GPU; the shell-volume normalisation runs there too,
in FP64, within a stated bound of the reference's numpy evaluation.  The
frames of the last trajectory stay resident between calls.

One deliberate difference: the reference passes debug=1 to Gofrt here
(positional `False, 1` = every, debug), which appends every histogram to a
file gofrt.dump in the working directory; nothing is written here.
"""
import numpy as np

from . import engine as _engine


def max_l(start, stop, tmax=0):
    """Lag length and number of origins of [start, stop) (pyanalisi/analysis.py:77-86)."""
    if tmax <= 0:
        tmax = (stop - start) // 2
    n_ave = stop - start - tmax
    if start >= stop:
        raise RuntimeError("start index must be less than the end index")
    if n_ave <= 0:
        tmax = stop - start - 1
        n_ave = 1
    return tmax, n_ave


def hist2gofr(gr_N, gr_dr, gr_0, gofr):
    """Divides each bin by its shell volume 4pi/3 (r+^3 - r-^3)
    (pyanalisi/analysis.py:101-105), with the same numpy operations."""
    rs_m = np.arange(gr_N) * gr_dr + gr_0
    rs_p = (np.arange(gr_N) + 1) * gr_dr + gr_0
    vols = 4 * np.pi / 3 * (rs_p ** 3 - rs_m ** 3)
    return gofr / vols


def _frames(traj):
    return (traj.get_positions_copy(), traj.get_box_copy(), traj.get_type_ids(),
            int(traj.get_ntypes()), bool(traj.is_triclinic()))


# The engine holding the frames of the last trajectory used, kept resident
# across calls: the notebook pattern of several compute_gofr calls on one
# trajectory copies its frames to the GPU once.  The key is the trajectory's
# data version (a process-wide counter, new for every trajectory built), so a
# different or rebuilt trajectory is uploaded again.
_resident = {"key": None, "engine": None, "traj": None}

# bound on the relative difference of the last compute_gofr result from the
# reference's own host evaluation (numpy hist2gofr on the same buffer); 0.0
# when the histogram itself was returned (bit for bit the reference's)
last_error_bound = 0.0


def _resident_engine(traj, device):
    version = traj.data_version() if hasattr(traj, "data_version") else id(traj)
    key = (version, int(device))
    if _resident["engine"] is None or _resident["key"] != key:
        release_resident()
        pos, boxes, tids, ntypes, tric = _frames(traj)
        eng = _engine.Engine(device)
        eng.set_frames(pos, boxes, tids, ntypes, triclinic=tric)
        _resident.update(key=key, engine=eng, traj=traj)
    return _resident["engine"]


def release_resident():
    """Frees the device copy of the last trajectory's frames."""
    eng = _resident.get("engine")
    if eng is not None:
        eng.close()
    _resident.update(key=None, engine=None, traj=None)


def compute_gofr(traj, startr, endr, nbin, start=0, stop=None, tmax=1, tskip=10, n_segments=1,
                 nthreads=1, return_histogram=False, device=0, density=False,
                 return_error_bound=False):
    """g(r,t) of a pyanalisi.Trajectory (this package's module) as
    Analysis.compute_gofr: one array, or a list of n_segments arrays, each the
    reference Gofrt buffer (shape (leff, ntypes(ntypes+1), nbin)) or its
    shell-volume normalisation.  The frames stay on the GPU between calls on
    the same trajectory, and the normalisation runs there in FP64.

    density=True also divides by each channel's pair density (a g(r,t) that
    tends to 1; self channels: a probability density of the displacement).
    The result's bound on the relative difference from the reference's host
    evaluation is in `last_error_bound`, or returned as (result, bound) with
    return_error_bound=True."""
    global last_error_bound
    if stop is None:
        stop = traj.get_nloaded_timesteps()
    nthreads = max(1, int(nthreads or 1))
    tmax, n_ave = max_l(start, stop, tmax)
    if n_segments < 1:
        raise IndexError(f"n_segments must be > 0 ({n_segments})")
    norm = "buffer" if return_histogram else ("density" if density else "shell")
    eng = _resident_engine(traj, device)
    if n_segments == 1:
        res, bound = eng.gofr(startr, endr, nbin, tmax, tskip, 1, n_ave, [start], norm=norm,
                              nparts=nthreads)
        res = res[0]
    else:
        segment_size = max(1, n_ave // n_segments)
        offsets = list(range(0, min(segment_size * n_segments, n_ave), segment_size))
        out, bound = eng.gofr(startr, endr, nbin, tmax, tskip, 1, segment_size,
                              [start + i for i in offsets], norm=norm, nparts=nthreads)
        res = [out[k] for k in range(len(offsets))]
    last_error_bound = bound
    return (res, bound) if return_error_bound else res
