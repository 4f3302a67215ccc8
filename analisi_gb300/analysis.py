"""The reference's Python g(r) conveniences on the GB300 engine.

Restates pyanalisi/analysis.py:77-86 (max_l), :101-105 (hist2gofr) and
:108-145 (Analysis.compute_gofr) -- equivalently pyanalisi/common.py:186-206
(analyze_gofr) -- for a trajectory of this package's `pyanalisi` module.
The segmented form (n_segments > 1), a loop of Gofrt::calculate calls in the
reference, runs every segment of the resident frames in one persistent
launch (gofr_run_windows).  Results carry the reference's exact doubles: the
counts of each reference thread partition are folded as its threads add incr.

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


def compute_gofr(traj, startr, endr, nbin, start=0, stop=None, tmax=1, tskip=10, n_segments=1,
                 nthreads=1, return_histogram=False, device=0):
    """g(r,t) of a pyanalisi.Trajectory (this package's module) as
    Analysis.compute_gofr: one array, or a list of n_segments arrays, each the
    reference Gofrt buffer (shape (leff, ntypes(ntypes+1), nbin)) or its
    shell-volume normalisation."""
    if stop is None:
        stop = traj.get_nloaded_timesteps()
    nthreads = max(1, int(nthreads or 1))
    tmax, n_ave = max_l(start, stop, tmax)
    pos, boxes, tids, ntypes, tric = _frames(traj)
    dr = (endr - startr) / nbin

    def finish(counts, n):
        parts = counts if nthreads > 1 else counts[None]
        buf = _engine.counts_to_buffer(parts, n, tskip, nparts=nthreads)
        return buf if return_histogram else hist2gofr(nbin, dr, startr, buf)

    with _engine.Engine(device) as eng:
        eng.set_frames(pos, boxes, tids, ntypes, triclinic=tric)
        if n_segments == 1:
            c = eng.run(startr, endr, nbin, tmax, tskip, 1, n_ave, start, nparts=nthreads)
            return finish(c, n_ave)
        if n_segments > 1:
            segment_size = max(1, n_ave // n_segments)
            offsets = list(range(0, min(segment_size * n_segments, n_ave), segment_size))
            c = eng.run_windows(startr, endr, nbin, tmax, tskip, 1, segment_size,
                                [start + i for i in offsets], nparts=nthreads)
            return [finish(c[k], segment_size) for k in range(len(offsets))]
    raise IndexError(f"n_segments must be > 0 ({n_segments})")
