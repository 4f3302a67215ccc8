/*
 * gofr_gb300.h -- C ABI of the GB300 (sm_103a) van Hove g(r,t) engine.
 *
 * This is the drop-in boundary for analisi's Gofrt calculation
 * (lib/include/gofrt.h, lib/src/gofrt.cpp).  The C++ Gofrt class of
 * analisi_gb300/host/gofrt.h and its Python binding call only these entry
 * points; any other language binds them with a plain FFI (ctypes, cgo, JNI).
 *
 * Conventions
 *   - Every entry point returns an int status: GOFR_OK (0) or a negative
 *     gofr_status.  No C++ exception ever crosses this boundary.
 *   - gofr_last_error(ctx) returns the message of the last failure on ctx.
 *   - One context owns one CUDA stream and the device-resident frames of one
 *     trajectory.  A context is thread-compatible, not thread-safe, like one
 *     reference Gofrt object (nothing in the reference is re-entrant).
 *   - Positions and boxes are the reference's INTERNAL buffers, i.e. what
 *     Trajectory_numpy / Trajectory hold after their preprocessing
 *     (lib/src/trajectory_numpy.cpp:7-199): positions [nframes][natoms][3]
 *     FP64, boxes [nframes][6 or 9] FP64 in the internal format
 *     {xlo, ylo, zlo, lx/2, ly/2, lz/2, xy, xz, yz}
 *     (lib/include/basetrajectory.h:21-43,94-105), dense type ids 0..ntypes-1
 *     (lib/src/basetrajectory.cpp:52-89).
 *   - Histogram counts are exact unsigned 64-bit integers laid out as the
 *     reference's result buffer: [leff][ntypes*(ntypes+1)][nbin]
 *     (lib/src/gofrt.cpp:65-71); lags not on the `every` grid stay 0.  The
 *     reference's double value of a bin is count * incr
 *     (incr = 1/int(ntimesteps/skip), lib/src/gofrt.cpp:91-92), or its exact
 *     thread-fold when per-partition counts are requested (nparts > 1).
 */
#ifndef GOFR_GB300_H
#define GOFR_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gofr_ctx gofr_ctx;

enum gofr_status {
    GOFR_OK = 0,
    GOFR_ERR_ARG = -1,      /* invalid argument (shape, null pointer, value) */
    GOFR_ERR_RANGE = -2,    /* leff+ntimesteps+primo > nframes+1 (reference: runtime_error, gofrt.cpp:81-83) */
    GOFR_ERR_CUDA = -3,     /* a CUDA runtime call failed */
    GOFR_ERR_NOMEM = -4,    /* device or host allocation failed */
    GOFR_ERR_STATE = -5,    /* no frames uploaded yet */
    GOFR_ERR_DEVICE = -6,   /* a kernel reported an error word (bounded wait ran out, wrap loop cap) */
    GOFR_ERR_UNSUPPORTED = -7,
    GOFR_ERR_NEIGH_FULL = -8  /* a neighbour list overflowed (reference: "Too many neighbours in
                                 shell!", lib/src/neighbour.cpp:44-47) */
};

enum gofr_box_kind {
    GOFR_BOX_ORTHO = 0,     /* box stride 6 (lib/include/basetrajectory.h:38-43) */
    GOFR_BOX_TRICLINIC = 1  /* box stride 9 (lib/include/basetrajectory.h:32-37) */
};

enum gofr_kernel {
    GOFR_KERNEL_AUTO = 0,        /* FP32 bulk + FP64 edge recheck when certifiable, else FP64;
                                    the cell-list form when its modelled time is lower */
    GOFR_KERNEL_F32_RECHECK = 1, /* force the all-pairs FP32 + recheck kernel (error if not
                                    certifiable) */
    GOFR_KERNEL_F64 = 2,         /* plain FP64 kernel: reference arithmetic for every pair */
    GOFR_KERNEL_CELL = 3,        /* cell-list FP32 + recheck kernel (error if not eligible);
                                    ANALISI_GB300_CELL_PLAN="reach,r,bx,by,bz" pins its
                                    configuration when that one is eligible */
    GOFR_KERNEL_TUNED = 4,       /* AUTO, but the kernel and its configuration are picked
                                    by timing them on a sample of the job: the all-pairs
                                    kernel, the block cell-list kernel (cell size, block
                                    shape, first atoms per thread) and the warp-streamed
                                    cell-list kernel (cell size, warp block shape, CTA
                                    size 8 or 16 warps, one or two copies of the shared
                                    histogram); the choice is
                                    remembered per key (log2 N, nbin, ntypes, box kind,
                                    cell grid) in the process and, when the environment
                                    variable ANALISI_GB300_TUNE_CACHE names a file, across
                                    runs; AUTO takes a remembered choice for its key
                                    (ANALISI_GB300_TUNE_LOG: a file for every timing) */
    GOFR_KERNEL_CELL_WARP = 5    /* warp-streamed cell-list FP32 + recheck kernel: each warp
                                    streams the neighbourhood of its own small block of cells;
                                    orthorhombic and triclinic boxes (error if not eligible:
                                    the cell-list conditions, a histogram and channel
                                    table that fit shared memory, and tilts
                                    that keep the images a block reaches within two box
                                    edges).  AUTO takes it wherever it would take the block
                                    cell-list form, and for a triclinic box when it
                                    evaluates under half of the pairs.
                                    ANALISI_GB300_CELLW_PLAN="reach,4,wx,wy,wz" pins its
                                    configuration (4: the records a lane holds) */
};

/* Parameters of one Gofrt::calculate (lib/include/gofrt.h:37-45 constructor
 * arguments, reset(n) and calculate(primo)). */
typedef struct gofr_params {
    double rmin;            /* Gofrt(..., rmin, ...) */
    double rmax;            /* Gofrt(..., rmax, ...) */
    unsigned nbin;          /* Gofrt(..., nbin, ...) */
    unsigned tmax;          /* Gofrt(..., tmax): maximum lag; 0 = ntimesteps */
    unsigned skip;          /* origin stride; 0 means 1 (calculatemultithread.h:44) */
    unsigned every;         /* lag stride; 0 means 1 (calculatemultithread.h:45) */
    unsigned ntimesteps;    /* reset(ntimesteps) */
    unsigned long long primo; /* calculate(primo) */
    int kernel;             /* enum gofr_kernel */
    unsigned nparts;        /* >1: counts per reference thread partition
                               (calculatemultithread.h:50-78), output is
                               [nparts][leff][nch][nbin]; 0/1: totals */
} gofr_params;

/* Statistics of the last run on a context. */
typedef struct gofr_stats {
    unsigned long long pairs;        /* ordered pairs of the reference loop (N^2 per lag/origin) */
    unsigned long long evaluated;    /* pairs whose distance was computed on the GPU */
    unsigned long long candidates;   /* FP32 pairs inside the accept window (+ its error bound) */
    unsigned long long rechecks;     /* pairs recomputed in FP64 */
    double kernel_ms;                /* device time of the pair kernel(s), CUDA events */
    double total_ms;                 /* device time of the whole run incl. copies */
    int kernel_used;                 /* enum gofr_kernel actually launched */
    int wrap_checked;                /* 1 if the per-pair wrap-decision check was on */
    double err_bound_d2;             /* FP32 error bound on d2 at rmax (A^2) */
    unsigned long long launches;     /* kernels launched on this context since its creation */
    unsigned long long h2d_bytes;    /* frame bytes copied host -> device since its creation */
} gofr_stats;

/* Creates a context on CUDA device `device` (replaces the construction of a
 * Gofrt object, lib/src/gofrt.cpp:22-31, whose work is per-call here). */
int gofr_ctx_create(gofr_ctx **out, int device);

/* Releases the context, its stream and all its device memory (the end of a
 * Gofrt object, Gofrt::~Gofrt, lib/src/gofrt.cpp:33). */
void gofr_ctx_destroy(gofr_ctx *ctx);

/* Message of the last error on ctx ("" if none); ctx may be NULL for
 * failures of gofr_ctx_create. */
const char *gofr_last_error(const gofr_ctx *ctx);

/* Copies one trajectory into HBM, where it stays resident for every later
 * run (replaces the per-pair host reads of Trajectory_numpy::positions/box,
 * lib/include/trajectory_numpy.h:19-23, and BaseTrajectory::get_type,
 * lib/include/basetrajectory.h:71-77).  The host buffers may be freed after
 * the call returns.  Pinned host memory makes the copy asynchronous-capable
 * and faster; pageable memory works too. */
int gofr_set_frames(gofr_ctx *ctx, const double *positions, const double *boxes,
                    int box_kind, const int *type_ids, unsigned ntypes,
                    size_t natoms, size_t nframes);

/* Number of unsigned 64-bit counts gofr_run writes for these parameters
 * (leff * ntypes*(ntypes+1) * nbin, times nparts when nparts > 1): the
 * product of Gofrt::get_shape, lib/src/gofrt.cpp:65-67. */
int gofr_output_size(const gofr_ctx *ctx, const gofr_params *p, size_t *n_counts);

/* One Gofrt::calculate(primo) on the resident frames (replaces
 * CalculateMultiThread::calculate, lib/include/calculatemultithread.h:106-162,
 * Gofrt::calc_init/calc_single_th/calc_end, lib/src/gofrt.cpp:74-155).
 * Writes exact counts into the caller's host buffer and returns when done. */
int gofr_run(gofr_ctx *ctx, const gofr_params *p, unsigned long long *counts_host);

/* Same as gofr_run (Gofrt::calculate, lib/src/gofrt.cpp:74-155), asynchronous:
 * counts go to a caller-owned device buffer of gofr_output_size elements,
 * work is queued on the context's stream.  Call gofr_sync before reading the
 * counts. */
int gofr_run_device(gofr_ctx *ctx, const gofr_params *p, unsigned long long *counts_device);

/* Waits for the context's stream and reports device-side errors (the join
 * that ends the reference's CalculateMultiThread::calculate,
 * lib/include/calculatemultithread.h:106-162, which is synchronous). */
int gofr_sync(gofr_ctx *ctx);

/* Several Gofrt::calculate windows of the resident frames in one persistent
 * launch: window w is calculate(primos[w]) with the parameters p (the segmented
 * loop of pyanalisi/analysis.py:131-142 and pyanalisi/common.py:196-203, or the
 * blocks of lib/include/blockaverage.h:107-190).  counts_host receives
 * [nwin][nparts][leff][nch][nbin] (nparts taken as 1 when p->nparts <= 1).
 * The FP32 kernel runs every (window, partition) in one launch; parameters
 * that need the FP64 or cell-list kernel run one launch per window. */
int gofr_run_windows(gofr_ctx *ctx, const gofr_params *p, unsigned nwin,
                     const unsigned long long *primos, unsigned long long *counts_host);

/* One or several Gofrt::calculate windows (as gofr_run_windows; nwin = 0 or
 * primos = NULL: one window, calculate(p->primo)) with the result made into
 * doubles on the GPU in FP64, out_host receiving [nwin][leff][nch][nbin]:
 *   norm 0: the reference's result buffer, bit for bit: each reference
 *           thread partition's bin is incr added count times, the partitions
 *           folded in order (lib/src/gofrt.cpp:118,127-132; nparts <= 1: one
 *           partition);
 *   norm 1: that buffer divided by the shell volume 4 pi/3 (r+^3 - r-^3),
 *           r- = b dr + rmin, r+ = (b+1) dr + rmin: the reference's Python
 *           hist2gofr (pyanalisi/analysis.py:101-105, the normalisation of
 *           Analysis.compute_gofr, :108-145);
 *   norm 2: norm 1 further divided by each channel's pair density (distinct
 *           pairs of types a != b: 2 N_a N_b / V, of one type a:
 *           N_a (N_a - 1) / V; the self channel of type a: N_a), V the box
 *           volume averaged over the windows' origin frames (no counterpart in
 *           the reference, which leaves this to the caller).
 * rel_err_bound (optional) receives a bound on the relative difference of any
 * element from the same formula evaluated on the host in FP64 with cubes
 * within one unit in the last place of exact (numpy's `r ** 3`): 0 for
 * norm 0.  The frames stay resident: only the doubles come back. */
int gofr_run_normalized(gofr_ctx *ctx, const gofr_params *p, unsigned nwin,
                      const unsigned long long *primos, int norm, double *out_host,
                      double *rel_err_bound);

/* One Gofrt::calculate(primo) (as gofr_run) on frames that stay in the
 * caller's host memory, for trajectories larger than the device should hold:
 * the reference bounds its memory the same way, with a window of frames
 * loaded at a time (Trajectory::set_data_access_block_size / set_access_at,
 * lib/src/trajectory.cpp:349-384,450-690).  The origins are split into chunks
 * whose frames (first origin to last origin + last lag) fit max_device_bytes;
 * each chunk's frames are copied to the device (replacing the context's
 * resident frames), run, and its exact counts added: the counts equal
 * gofr_run's on the whole trajectory.  Arguments as gofr_set_frames and
 * gofr_run; GOFR_ERR_UNSUPPORTED when the budget cannot hold one origin's
 * lags. */
int gofr_run_streamed(gofr_ctx *ctx, const double *positions, const double *boxes, int box_kind,
                      const int *type_ids, unsigned ntypes, size_t natoms, size_t nframes,
                      const gofr_params *p, size_t max_device_bytes,
                      unsigned long long *counts_host);

/* Statistics of the last completed run.  No reference counterpart: the
 * reference reports no per-run statistics. */
int gofr_get_stats(const gofr_ctx *ctx, gofr_stats *out);

/* Converts counts to the reference's double result buffer, with
 * incr = 1/int(ntimesteps/skip) (gofrt.cpp:91-92).  nparts >= 1: counts are
 * [nparts][n] per reference thread partition and the result is the
 * reference's exact value: each partition's bin is incr added count times in
 * sequence (gofrt.cpp:118), partitions folded in order (gofrt.cpp:128-132).
 * nparts == 0: counts are [n] totals and out[i] = counts[i] * incr.
 * n is the number of doubles (leff*nch*nbin). */
int gofr_counts_to_buffer(const unsigned long long *counts, size_t n, unsigned nparts,
                          unsigned ntimesteps, unsigned skip, double *out);

/* Exact squared-distance bin thresholds used by the kernels: th[b] is the
 * smallest double d2 whose reference bin is >= b inside the accepted window,
 * th[0] the smallest accepted d2, th[nbin] the successor of the largest
 * accepted d2 (lib/src/gofrt.cpp:104,114-118).  th has nbin+1 doubles.
 * Returns GOFR_ERR_UNSUPPORTED when the bin map is not monotone
 * (rmax <= rmin, non-finite values). */
int gofr_bin_thresholds(double rmin, double rmax, unsigned nbin, double *th);

/* The plan gofr_run's planner takes (host only, no device, tuner cache not
 * consulted) for frames in one box (internal format, the same in every
 * frame) with coordinates within [coord_min, coord_max] per axis, natoms
 * atoms of ntypes types and parameters p (p->kernel as for gofr_run).  out
 * (10 ints): [0] the kernel (GOFR_KERNEL_F32_RECHECK, _F64, _CELL or
 * _CELL_WARP), [1] the cell reach, [2..4] cells per axis, [5..7] the
 * (warp) block of cells, [8] warps per CTA of the warp-streamed kernel, [9] 1
 * when the all-pairs kernel needs its per-pair wrap check; cell fields 0 for
 * the all-pairs kernels.  Returns the status gofr_run would (e.g.
 * GOFR_ERR_UNSUPPORTED for a forced cell-list kernel the box cannot take).
 * No reference counterpart (the reference has one pair loop,
 * lib/src/gofrt.cpp:96-122): it shows the planner's choices without a GPU. */
int gofr_plan_query(const double *box, int box_kind, const double *coord_min,
                    const double *coord_max, size_t natoms, unsigned ntypes,
                    const gofr_params *p, int *out);

/* Neighbourhood tables of the warp-streamed cell-list kernel (host only, no
 * device work) for one box (internal format, 6 or 9 doubles), the
 * coordinates' extent per axis [coord_min, coord_max], rmax and a cell grid
 * nc[3]: the ranges a warp block of cells [c0, c0 + cn) reaches, relative to
 * it, per lattice image.  tables (38 ints): layers uz in [cz0 + t[0],
 * cz0 + cnz + t[1]]; in a layer of image sz (-1..1), rows uy in
 * [cy0 + t[2 + sz + 1], cy0 + cny + t[5 + sz + 1]]; in a row of images
 * (sy, sz), cells ux in [cx0 + t[8 + k], cx0 + cnx + t[23 + k]],
 * k = (sz + 1) 5 + sy + 2 (images s = floor(u / nc)).  shifts (75 x 3
 * floats, optional): the FP32 lattice vector of image (sx, sy, sz) at
 * (sx + 2) + 5 (sy + 2) + 25 (sz + 1).  bound (3 doubles, optional): the
 * certified per-axis error e_k of the kernel's FP32 difference components
 * against the reference's FP64 ones, from which the windows follow
 * (|d2_f32 - d2_ref| <= (2 sqrt(d2) |e| + 2 |e|^2 + 5.01 2^-24 d2)(1 + 2^-20)).
 * Returns GOFR_ERR_UNSUPPORTED when an
 * image falls outside the table (the kernel then refuses the box).  No
 * reference counterpart: the reference evaluates every pair
 * (lib/src/gofrt.cpp:101-102); this exposes the cell-list geometry so that
 * its completeness can be checked without a GPU. */
int gofr_cellw_tables(const double *box, int box_kind, const double *coord_min,
                      const double *coord_max, double rmax, const int *nc, int *tables,
                      float *shifts, double *bound);

/* Measures, on `device`, the two peaks that bound the FP32 pair kernel: the
 * FP32 lane-operation rate (one FFMA = one operation, the unit of the kernel's
 * 16/19 operations per pair) and the shared-memory u32 atomic rate.  No
 * reference counterpart: the reference has no GPU path. */
int gofr_measure_peaks(int device, double *fp32_lane_ops_per_s, double *smem_atomics_per_s);

/* Allocation-free variant of the plain FP64 pair kernel.  No counterpart in
 * the reference (whose calculation never touches a GPU).
 *
 * For callers that cannot call cudaMalloc: code running under a framework
 * that owns all device memory through its own pool, a real-time loop that
 * must not allocate, or a plug-in whose host has laid out every device byte
 * already.  The caller passes its own DEVICE buffers: positions
 * [nframes][natoms][3] and boxes [nframes][6 or 9] in the reference's internal
 * format (as for gofr_set_frames), type ids [natoms] in 0..ntypes-1, and the
 * output counts [leff][ntypes*(ntypes+1)][nbin] (zeroed here).  boxes and the
 * type ids are read on the device only: an id outside 0..ntypes-1 is found
 * there, its atom's pairs are skipped and the call returns GOFR_ERR_DEVICE
 * with a type-id message.  The same exact counts as gofr_run with
 * GOFR_KERNEL_F64.
 *
 * Nothing is allocated: the only scratch (channel table, error word) is a
 * file-scope __device__ array of 768 bytes that every GPU loading this library
 * holds until the process exits.  Limits: ntypes <= 16, nparts <= 1, and the
 * shared-memory histogram of ntypes*(ntypes+1)*nbin u32 must fit one CTA.
 * p->kernel is ignored.  Work runs on `stream` (a cudaStream_t; NULL = the
 * legacy default stream) of the current device; the call waits for it and
 * returns the kernel's error status.  The first call on a device resolves the
 * scratch array's device address (cudaGetSymbolAddress): make that first
 * call before any stream capture on that device.  All calls share the one
 * scratch array, so calls that overlap on the GPU (several host threads or
 * streams at once) race and must be serialised by the caller.  errbuf
 * (optional, errlen bytes) receives the message of a failure. */
int gofr_run_f64_noalloc(const double *d_positions, const double *d_boxes, int box_kind,
                         const int *d_type_ids, unsigned ntypes, size_t natoms, size_t nframes,
                         const gofr_params *p, unsigned long long *d_counts, void *stream,
                         char *errbuf, size_t errlen);

/* ---- batched trajectories (one persistent launch) --------------------- */

/* Description of one trajectory of a batch.  Pointers are host buffers in
 * the same internal format as gofr_set_frames. */
typedef struct gofr_traj_desc {
    const double *positions;
    const double *boxes;
    int box_kind;
    const int *type_ids;
    unsigned ntypes;
    size_t natoms;
    size_t nframes;
    gofr_params params;      /* per-trajectory parameters (kernel and nparts ignored) */
} gofr_traj_desc;

/* Uploads a batch of trajectories to a context (replacing any frames).  The
 * reference runs one Gofrt per trajectory (lib/src/gofrt.cpp:22-31 per object,
 * the caller's loop, e.g. pyanalisi/common.py:196-203); a batch replaces that
 * loop. */
int gofr_batch_set(gofr_ctx *ctx, const gofr_traj_desc *trajs, unsigned ntraj);

/* Number of counts of trajectory k of the current batch (Gofrt::get_shape,
 * lib/src/gofrt.cpp:65-67, of that trajectory), and its offset in the
 * concatenated output of gofr_batch_run. */
int gofr_batch_output_layout(const gofr_ctx *ctx, unsigned k, size_t *offset, size_t *n_counts);

/* One Gofrt::calculate (lib/src/gofrt.cpp:74-155) per trajectory of the
 * batch, all in one persistent launch that pulls
 * (trajectory, origin, lag, tile) items from a device work queue.  With
 * use_graph != 0 the launch sequence is captured once into a CUDA graph and
 * replayed.  counts_host receives the concatenation of every trajectory's
 * [leff][nch][nbin] counts (gofr_batch_output_layout gives the offsets). */
int gofr_batch_run(gofr_ctx *ctx, int use_graph, unsigned long long *counts_host);

/* ------------------------------------------------------------------------
 * Mean square displacement on the resident frames (the reference's
 * MSD<T>, lib/include/msd.h:25-58, lib/src/msd.cpp:24-118).
 * ------------------------------------------------------------------------ */

/* MSD(t, skip, tmax, nthreads, calcola_msd_centro_di_massa,
 * calcola_msd_nel_sistema_del_centro_di_massa, debug) + reset(ntimesteps) +
 * calculate(primo). */
typedef struct gofr_msd_params {
    unsigned skip;                 /* origin stride (0 means 1) */
    unsigned tmax;                 /* lmax: lags 0..leff-1, leff = min(ntimesteps, tmax) (0: ntimesteps) */
    unsigned ntimesteps;           /* reset(n): origins primo + k skip, k skip < n */
    unsigned long long primo;      /* calculate(primo) */
    int center_of_mass;            /* also the MSD of each type's centre of mass (f_cm = 2) */
    int in_center_of_mass_frame;   /* atomic displacements minus their type's centre-of-mass
                                      displacement */
} gofr_msd_params;

/* Per-frame, per-type centres of mass [nframes][ntypes][3] FP64 as the
 * reference's Trajectory_numpy::calc_cm_pos_vel computes them
 * (lib/src/trajectory_numpy.cpp:201-222: running mean over the atoms of each
 * type of the caller's positions); needed only for the two centre-of-mass
 * options.  nframes and ntypes must match the uploaded frames. */
int gofr_set_centres(gofr_ctx *ctx, const double *centres, size_t nframes, unsigned ntypes);

/* Number of doubles of the MSD result: leff * (center_of_mass ? 2 : 1) * ntypes,
 * the product of MSD::get_shape, lib/include/msd.h:38. */
int gofr_msd_output_size(const gofr_ctx *ctx, const gofr_msd_params *p, size_t *n);

/* Runs MSD::calculate(primo) on the resident frames (positions as they are,
 * no minimum image, like the reference's positions<false>) and writes the
 * result [leff][f_cm][ntypes] to out_host (double).  Element (t, 0, k) is the
 * mean over origins and atoms of type k of |x(o) - x(o+t)|^2 (optionally
 * minus the type's centre-of-mass displacement); (t, 1, k) the mean over
 * origins of the centre-of-mass |cm_k(o) - cm_k(o+t)|^2.  Each displacement is
 * the reference's FP64 value; its squared components are added into FP64 sums
 * (fused multiply-adds, a fixed order) divided by the count, where the
 * reference keeps a running mean: the two agree to rounding (relative ~1e-13
 * for 1e7 terms).  Errors as
 * lib/src/msd.cpp:57-68 (GOFR_ERR_RANGE: trajectory too short). */
int gofr_msd_run(gofr_ctx *ctx, const gofr_msd_params *p, double *out_host);

/* ------------------------------------------------------------------------
 * Neighbour lists of one resident frame (the reference's Neighbours<T,double>,
 * lib/include/neighbour.h:9-104, lib/src/neighbour.cpp:9-97).
 * ------------------------------------------------------------------------ */

/* One entry of the reference's ListSpec: (max neighbours, cutoff^2, skin^2)
 * for neighbours of one type (the skin is not used by the list build). */
typedef struct gofr_neigh_spec {
    unsigned long long nneigh;
    double cut2;
    double skin2;
} gofr_neigh_spec;

/* Lengths of the reference's two arrays for these specs (one per type), as
 * the Neighbours constructor sizes them (lib/include/neighbour.h:31-46):
 * list  natoms * (sum nneigh + ntypes) u64: per type k from
 *       list_off[k] = sum_{k'<k} (nneigh[k'] + 1) natoms, per atom i at
 *       list_off[k] + i (nneigh[k] + 1): the list size, then the indices;
 * rpos  natoms * 4 * sum nneigh doubles: from rpos_off[k] = sum_{k'<k}
 *       nneigh[k'] natoms 4, per atom at rpos_off[k] + i nneigh[k] 4:
 *       {r, x, y, z} per neighbour, x = x_i - x_neighbour (minimum image). */
int gofr_neigh_layout(const gofr_ctx *ctx, const gofr_neigh_spec *spec, unsigned nspec,
                      size_t *list_len, size_t *rpos_len);

/* Neighbours::update_neigh(timestep, sort), lib/src/neighbour.cpp:9-79, with
 * the sort of lib/src/neighbour.cpp:49-78, on the resident frame `timestep`:
 * for every atom and neighbour type, the atoms of that type within its cutoff
 * (d2 <= cut2 of the neighbour's type, FP64 minimum image as the reference),
 * in ascending index order, or sorted by distance when sort != 0 (stable);
 * list_host / rpos_host receive the arrays above (entries past a list's size
 * are 0).  A pair within either type's cutoff that finds one of the two lists
 * full is the reference's error: GOFR_ERR_NEIGH_FULL, with the reference's
 * message (iatom, jatom, ni, nj, itype, jtype of the first such pair in its
 * loop order) in gofr_last_error.  At most 32 types. */
int gofr_neigh_run(gofr_ctx *ctx, const gofr_neigh_spec *spec, unsigned nspec, size_t timestep,
                   int sort, unsigned long long *list_host, double *rpos_host);

#ifdef __cplusplus
}
#endif

#endif /* GOFR_GB300_H */
