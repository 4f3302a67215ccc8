// Internal declarations shared by the host side (gofr_capi.cu) and the
// kernels (gofr_kernels.cu).  Not part of the C ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace gofr {

// Bits of the device error word.
enum : unsigned {
    ERRW_WAIT_TIMEOUT = 1u,   // a bounded mbarrier wait ran out
    ERRW_WRAP_LOOP = 2u,      // the FP64 iterative minimum image exceeded its iteration cap
    ERRW_QUEUE = 4u,          // a work queue overflowed its capacity
    ERRW_BOUNDS = 8u,         // a bounds check failed (GOFR_CHECK in GOFR_DEBUG_BOUNDS builds;
                              // the warp-streamed kernel's neighbourhood tables always)
    ERRW_HIST_OVERFLOW = 16u  // an item could have overflowed a u32 shared bin (run discarded)
};

// Debug builds (-DGOFR_DEBUG_BOUNDS): GOFR_CHECK(cond, err) records a failed
// index check in the error word (no trap) and is false, so the access it
// guards is skipped; in normal builds it is `true` and costs nothing.
#ifdef GOFR_DEBUG_BOUNDS
#define GOFR_CHECK(cond, err) ((cond) ? true : (atomicOr((err), (unsigned)ERRW_BOUNDS), false))
#else
#define GOFR_CHECK(cond, err) true
#endif

// Stats slots (unsigned long long) on the device.
enum : int { ST_CANDIDATES = 0, ST_RECHECKS = 1, ST_EVALUATED = 2, ST_COUNT = 4 };

// Per-frame FP32 box parameters for the FP32 kernels (12 floats, 48 B).
//   L[3]    full edges 2*lh rounded to float
//   invL[3] 1/(2*lh) rounded to float
//   tilt[3] {xy, xz, yz} rounded to float
struct Box32 {
    float L[3];
    float invL[3];
    float tilt[3];
    float pad[3];
};

// One launch of an all-pairs kernel over (lag, i-tile, origin) items.
struct PairLaunch {
    const float *pos32;       // [T][3][NP] SoA {x-cx | y-cy | z-cz}, padding NaN
    const unsigned char *types8; // [NP] dense type ids (padding 0)
    const double *pos64;      // [T][N][3] internal FP64 positions (reference values)
    const double *box64;      // [T][9] internal boxes (tilts zero when orthorhombic)
    const Box32 *box32;       // [T]
    const float2 *win;        // [nbin] certified FP32 window {lo, hi} of each bin
    const unsigned short *chtab; // [ntypes*ntypes] channel of a type pair
    unsigned long long *counts;  // [leff][nch][nbin]
    unsigned *err;
    unsigned long long *stats;
    int N, NP, nbin, nch, ntypes;
    int a0, a1;               // first-atom range [a0, a1) (one reference thread partition)
    int n_lags, every;        // lags t = l*every, l < n_lags
    int n_orig, skip;         // origins primo + k*skip, k < n_orig
    long long primo;
    int n_itiles;             // tiles of the first-atom range
    long long n_items;        // n_lags * n_itiles * n_orig
    float hi_f, lo_f;         // certain reject above hi_f / below lo_f
    float rmin_f, inv_dr_f;   // bin guess
    float wlim;               // wrap check: |frac| > wlim flags a recheck
    double rmin, rmax, dr, rmin2, rmax2;  // reference binning constants
    int tric;
    int wchk;                 // batched kernel: per-pair wrap-decision check on
    int ghist;                // histogram too large for shared memory: atomics go
                              // straight to the u64 counts in global memory
    int dbg_stall;            // GOFR_DEBUG_BOUNDS builds only: the first tile's
                              // barrier expects bytes that no copy brings, so the
                              // bounded wait runs out (test of that path)
};

// One work descriptor of the batched kernel: origins [k0, k1) of one
// (trajectory, lag, first-atom tile).
struct WorkDesc {
    int traj, lag_idx, itile, k0, k1, pad0, pad1, pad2;
};

// One launch of the cell-list pair kernel (gofr_cells.cu): items are
// (lag, block of cells, origin), pair.n_items = n_lags * nblocks * n_orig.
struct CellLaunch {
    PairLaunch pair;
    const int *start;              // [T][ncell+1] sorted-atom offset of each cell
    const float *spos;             // [T][3][NP] FP32 frames sorted by cell
    const unsigned *sidt;          // [T][NP] type << 24 | original atom id of each sorted slot
    int nc[3];                     // cells per axis
    int b[3];                      // cells per block per axis
    int nb[3];                     // blocks per axis
    int reach;                     // neighbour cells per side (cell edge >= rmax / reach)
    int r;                         // first atoms per thread (2, 3 or 4)
};

// One launch of the warp-streamed cell-list kernel (gofr_cellw.cu): items
// are (lag, origin, part), pair.n_items = n_lags * n_orig * parts; each warp
// takes blocks of w[0] x w[1] x w[2] cells of the part's range.
//
// Cells are an axis-aligned grid of the box [lo, lo + L) (triclinic: the
// upper-triangular cell's axis-aligned fundamental domain).  A warp block's
// neighbourhood is given relative to the block, per lattice image
// (sx, sy, sz) of the cells reached: layers uz in [cz0 + nz_lo, cz0 + cnz +
// nz_hi] (image sz = floor(uz / ncz)); in a layer of image sz, rows uy in
// [cy0 + ny_lo[sz+1], cy0 + cny + ny_hi[sz+1]] (image sy); in a row of images
// (sy, sz), cells ux in [cx0 + nx_lo[k], cx0 + cnx + nx_hi[k]], k = (sz + 1) 5 +
// sy + 2 (image sx).  Orthorhombic boxes have lo = -reach, hi = reach - 1
// everywhere; a triclinic layer or row is shifted by the tilts, so its range
// starts a fraction of a cell off and may take one cell more.  shift[]
// holds the FP32 lattice vector of each image, index (sx + 2) + 5 (sy + 2) +
// 25 (sz + 1).
constexpr int CELLW_MAX_ROWS = 64;  // neighbourhood rows of a warp block (all its layers)
constexpr int CELLW_NSHIFT = 75;    // images sx, sy in -2..2, sz in -1..1
constexpr int CELLW_SHIFT0 = 37;    // index of the image (0, 0, 0)
struct CellwLaunch {
    PairLaunch pair;
    const int *start;              // [T][ncell+1] sorted-record offset of each cell
    const float4 *wpos;            // [T][NP] {x, y, z, type << 24 | atom id} sorted by cell
    int nc[3];                     // cells per axis
    int w[3];                      // cells per warp block per axis
    int nw[3];                     // warp blocks per axis
    int reach;                     // neighbour cells per side
    int r;                         // records per lane (4; kept in plans and tuner keys)
    int parts;                     // parts of the warp blocks per (lag, origin)
    int cta_warps;                 // warps per CTA: 8 (two CTAs per SM) or 16 (one)
    int hcopy;                     // copies of the shared histogram (privatisation depth: 1, 2)
    int nz_lo, nz_hi;              // neighbourhood layers (see above)
    int ny_lo[3], ny_hi[3];        // rows, per layer image sz + 1
    int nx_lo[15], nx_hi[15];      // cells, per row images (sz + 1) 5 + sy + 2
    int ny_span;                   // max over sz of ny_hi - ny_lo + 1
    float4 shift[CELLW_NSHIFT];    // FP32 lattice vector {x, y, z, 0} of each image
};
int cellw_smem_bytes(int nch, int nbin, int ntypes, int cta_warps = 8, int hcopy = 1);
int cellw_chunk_records();  // neighbour records per chunk (4 per lane)
int cellw_batch_atoms();    // first atoms per batch (each batch streams the neighbourhood)
int cellw_chunk_pieces();   // bulk copies per chunk at most
// box_internal {xlo, ylo, zlo, lx/2, ly/2, lz/2, xy, xz, yz}; tric: the
// coordinates are reduced into the axis-aligned cell by the lattice (z, then
// y, then x), else per axis.
int launch_cell_scatter_w(const double *pos64, const unsigned char *types8, size_t T, size_t N,
                          const double *box_internal, const double *centre, const int *nc,
                          bool tric, const int *cell_of, const int *rank_of, const int *start,
                          float4 *wpos, cudaStream_t s);
int launch_cellw_pairs(const CellwLaunch &C, int num_sms, cudaStream_t s);

// FP64 normalisation of window counts on the device (gofr_norm.cu).
struct NormLaunch {
    const unsigned long long *counts;  // [nwin][nparts][n] exact counts
    double *out;                       // [nwin][n]
    const double *chfac;               // [nch] pair-density factors (mode 2)
    size_t n;                          // leff * nch * nbin
    int nwin, nparts, nbin, nch;
    int mode;                          // 0 buffer, 1 / shell volume, 2 / shell volume / density
    double incr;                       // 1 / int(ntimesteps / skip)
    double r0, dr;                     // bin b spans [b dr + r0, (b + 1) dr + r0)
    double c43pi;                      // fl(fl(4 pi) / 3)
};
int launch_counts_to_gofr(const NormLaunch &L, int num_sms, cudaStream_t s);

int cell_smem_bytes(int nch, int nbin, int ntypes);
int cell_block_atoms(int r);
int cell_max_ranges();
// Mean square displacement (gofr_msd.cu)
struct MsdLaunch {
    const double *pos64;    // [T][N][3]
    const double *cm;       // [T][ntypes][3] centres of mass (or null)
    const int *perm;        // [N] atom ids sorted by type (stable)
    const int *tbegin;      // [ntypes + 1] start of each type in perm
    double *partial;        // [leff][n_orig][f_cm * ntypes] sums over atoms
    int N, ntypes, leff, n_orig, skip;
    long long primo;
    int cm_msd, cm_self;
};
int launch_msd(const MsdLaunch &M, double *out_device, int num_sms, cudaStream_t s);

// Neighbour lists (gofr_neigh.cu)
constexpr int NEIGH_MAXT = 32;
struct NeighLaunch {
    const double *pos64;                  // [T][N][3]
    const double *box64;                  // [T][9] internal boxes
    const int *types;                     // [N] dense type ids
    const unsigned long long *nneigh;     // [ntypes] list capacities
    const unsigned long long *loff, *roff;  // [ntypes] offsets in list / rpos
    const double *cut2;                   // [ntypes] cutoffs^2
    unsigned long long *list;             // the reference's list array
    double *rpos;                         // the reference's rpos array
    int *full;                            // [N][ntypes] neighbour that filled a list (N: not full)
    unsigned *flags;                      // bit 0: some list is full; bit 1: a cell
                                          // neighbourhood held too many candidates
    unsigned long long *first_err;        // min i*N + j over overflowing pairs
    unsigned *err;                        // error word (minimum-image iteration cap)
    int N, ntypes;
    long long timestep;
    int tric;
    // FP32 prefilter (the all-pairs kernel's certified arithmetic): a pair
    // with d2_f32 > hi_f has reference d2 > the largest cutoff
    int prefilter;
    const float *pos32;                   // [T][3][NP]
    const Box32 *box32;                   // [T]
    long long NP;
    float hi_f;
    // cell-list form (orthorhombic boxes, prefilter on): the frame's cells of
    // edge >= the largest cutoff, at least 3 per axis
    int cells;
    int nc[3];
    const int *cstart;                    // [ncell + 1] first sorted slot of each cell
    const unsigned *csidt;                // [N] type << 24 | atom id in cell order
};
int launch_neigh_build(const NeighLaunch &L, int num_sms, cudaStream_t s);
int launch_neigh_check(const NeighLaunch &L, int num_sms, cudaStream_t s);
int launch_neigh_sort(const NeighLaunch &L, int num_sms, cudaStream_t s);

// Cell assignment and per-frame cell starts (and, with spos/sidt non-null,
// the block kernel's SoA sorted frames); cell_of and rank_of are left for
// launch_cell_scatter_w.  tric: cells of the coordinates reduced into the
// axis-aligned cell by the lattice (spos/sidt must then be null).
int launch_cell_build(const double *pos64, const unsigned char *types8, size_t T, size_t N,
                      const double *box_internal, const double *centre, const int *nc, bool tric,
                      int *cell_of, int *rank_of, int *count, int *start, float *spos,
                      unsigned *sidt, cudaStream_t s);
// One trajectory's cell-list items in one launch.
int launch_cell_pairs(const CellLaunch &C, int num_sms, cudaStream_t s);
// One launch over the items of nmem trajectories: Cs[m] (device) holds
// trajectory m's parameters, item_end[m] (device) the end of its items in the
// global item order; shared memory is sized for the largest histogram.
// prepare_* sets the kernel attributes and the grid (outside graph capture).
int prepare_cell_pairs_multi(int r, int max_nbin, int max_nch, int max_ntypes, int num_sms,
                             long long total, int *grid);
int launch_cell_pairs_multi(const CellLaunch *d_cells, const long long *d_end, int nmem,
                            int r, int max_nbin, int max_nch, int max_ntypes, int grid,
                            cudaStream_t s);

// Launch configuration helpers implemented in gofr_kernels.cu.
int launch_minmax(const double *pos64, size_t n3, double *d_out6, unsigned *d_nonfinite,
                  cudaStream_t s);
// Padded per-frame stride of the FP32 SoA frames.
inline size_t padded_natoms(size_t N) { return (N + 15) / 16 * 16; }
int launch_convert(const double *pos64, const int *types, size_t T, size_t N, double cx,
                   double cy, double cz, float *pos32, unsigned char *types8, cudaStream_t s);
// kind: 0 = FP32+recheck, 1 = FP64.  wrapcheck only for kind 0.
int launch_pairs(const PairLaunch &P, int kind, bool wrapcheck, int num_sms, cudaStream_t s,
                 size_t *smem_bytes_out);
int pairs_smem_bytes(int kind, int nch, int nbin, int ntypes, bool ghist = false);
int pairs_tile_atoms(int kind);
int batch_smem_bytes(int max_nbin, int max_nch, int max_ntypes);
int prepare_batch(int max_nbin, int max_nch, int max_ntypes, bool tric, int num_sms, int n_work,
                  int *grid_out);
int launch_batch_grid(const PairLaunch *d_trajs, const WorkDesc *d_work, int n_work,
                      unsigned *d_head, int max_nbin, int max_nch, int max_ntypes, bool tric,
                      unsigned *d_err, unsigned long long *d_stats, int grid, cudaStream_t s);
int launch_zero_u64(unsigned long long *p, size_t n, cudaStream_t s);

}  // namespace gofr
