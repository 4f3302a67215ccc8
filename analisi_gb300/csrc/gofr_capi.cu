// C ABI of the GB300 Gofrt engine (declared in include/gofr_gb300.h).
//
// Host-side responsibilities:
//   * frame residency: the reference's internal FP64 buffers are copied once
//     into HBM and converted there to FP32 {x,y,z,type} records;
//   * calc_init semantics (lib/src/gofrt.cpp:41-93): leff, the trajectory
//     length check, origins/lags grid, incr;
//   * exact bin thresholds in d2 space (gofr_bin_thresholds) and the certified
//     FP32 error bound that turns them into FP32 windows (certify());
//   * kernel selection (the planner's cost models, the cell grids and the
//     warp-streamed kernel's neighbourhood geometry, orthorhombic and
//     triclinic, with their certified bounds; the autotuner), launches,
//     counts back to the caller;
//   * the reference's double result buffer from counts, including its exact
//     per-thread fold (gofr_counts_to_buffer).
#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gofr_gb300.h"
#include "gofr_internal.h"

using namespace gofr;

namespace {

struct BoxStats {
    double Lmin[3], Lmax[3];   // full edges 2*lh over all frames
    double eL[3];              // max |fl32(L) - L|
    double tmax[3];            // max |tilt| {xy, xz, yz}
    double eT[3];              // max |fl32(tilt) - tilt|
    double lh_min;             // min half edge over frames and axes
};

struct TrajDev {
    size_t T = 0, N = 0;
    unsigned ntypes = 0;
    int tric = 0;
    double *pos64 = nullptr;
    float *pos32 = nullptr;          // [T][3][NP]
    unsigned char *types8 = nullptr; // [NP]
    double *box64 = nullptr;
    Box32 *box32 = nullptr;
    int *types = nullptr;
    std::vector<double> h_box;  // [T][9]
    double shift[3] = {0, 0, 0};
    double M[3] = {0, 0, 0};    // bound on |fl64(x - shift)| per axis
    BoxStats bs{};
    gofr_params params{};       // batch parameters
    size_t out_offset = 0, out_count = 0;
    bool box_constant = true;   // every frame has the same box
    // cell lists (built on first use for a grid, kept while the frames stay)
    int cell_nc[3] = {0, 0, 0};
    int *d_cstart = nullptr;
    unsigned *d_sidt = nullptr;
    float *d_spos = nullptr;
    float4 *d_wpos = nullptr;        // AoS sorted records of the warp-streamed kernel
    // MSD: atoms sorted by type, type starts, optional centres of mass
    std::vector<int> h_perm, h_tbegin, h_types;
    int *d_perm = nullptr, *d_tbegin = nullptr;
    double *d_cm = nullptr;          // [T][ntypes][3]
};

}  // namespace

struct gofr_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<TrajDev> trajs;
    unsigned long long *d_counts = nullptr;
    size_t cap_counts = 0;
    float2 *d_win = nullptr;
    size_t cap_win = 0;
    unsigned short *d_chtab = nullptr;
    size_t cap_chtab = 0;
    unsigned *d_err = nullptr;
    unsigned long long *d_stats = nullptr;
    double *d_msd_partial = nullptr, *d_msd_out = nullptr;
    size_t cap_msd_partial = 0, cap_msd_out = 0;
    // neighbour lists
    unsigned long long *d_nl_list = nullptr, *d_nl_meta = nullptr;
    double *d_nl_rpos = nullptr, *d_nl_cut2 = nullptr;
    int *d_nl_full = nullptr;

    size_t cap_nl_list = 0, cap_nl_meta = 0, cap_nl_rpos = 0, cap_nl_cut2 = 0, cap_nl_full = 0;
    double *d_minmax = nullptr;
    unsigned *d_nonfinite = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // a second stream for the batch's warp-streamed cell-list members, forked
    // from and joined back into `stream` (also inside a captured graph)
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    gofr_stats stats{};
    unsigned long long h2d_bytes = 0;  // bytes copied host -> device since creation
    double *d_gofr = nullptr;           // normalised results (gofr_run_normalized)
    size_t cap_gofr = 0;
    double *d_chfac = nullptr;
    size_t cap_chfac = 0;
    size_t batch_total = 0;
    unsigned long long launches = 0;  // kernels launched on this context
    // batched trajectories (gofr_batch_set / gofr_batch_run)
    struct Batch {
        std::vector<PairLaunch> launches;       // one per trajectory (FP32 path)
        std::vector<WorkDesc> work[2];          // descriptors, orthorhombic / triclinic
        std::vector<int> f64_trajs;             // trajectories that need the FP64 kernel
        int max_nbin = 1, max_nch = 1, max_ntypes = 1;
        PairLaunch *d_launches = nullptr;
        WorkDesc *d_work[2] = {nullptr, nullptr};
        unsigned *d_head = nullptr;             // queue heads [2]
        float2 *d_win = nullptr;
        unsigned short *d_chtab = nullptr;
        unsigned long long *h_stage = nullptr;  // pinned copy of the counts
        unsigned long long *d_counts = nullptr; // concatenated counts of every trajectory
        unsigned long long pairs = 0;
        int grid[2] = {0, 0};
        cudaGraphExec_t graph = nullptr;
        // members run through the cell-list kernel (one launch for all of them)
        std::vector<int> cell_trajs;
        std::vector<CellLaunch> cells;
        CellLaunch *d_cells = nullptr;
        long long *d_cell_end = nullptr;
        long long cell_items = 0;
        // members run by the warp-streamed cell-list kernel, one launch each,
        // largest first, on the second stream
        std::vector<CellwLaunch> cellw;
        unsigned long long allpairs_pairs = 0;  // pairs of the members not run with cells
        int cell_r = 3, cell_max_nbin = 1, cell_max_nch = 1, cell_max_ntypes = 1, cell_grid = 0;
    } batch;
};

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
namespace {

int fail(gofr_ctx *ctx, int code, const char *fmt, ...)
{
    if (ctx) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

#define CK(call)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? GOFR_ERR_NOMEM : GOFR_ERR_CUDA, \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                     \
    } while (0)

// Every device allocation of this file goes through here.  Fault-injection
// hook for tests: with ANALISI_GB300_FAIL_ALLOC=1 in the environment every
// allocation fails as if the device were out of memory, with
// ANALISI_GB300_FAIL_ALLOC=<tag> only the allocations made with that tag
// (e.g. "cells": the cell-sorted frames), so that the error paths and the
// fallbacks can be run without a real shortage; they must leave the context
// usable.
template <class T>
cudaError_t dev_malloc(T **p, size_t bytes, const char *tag = nullptr)
{
    const char *e = std::getenv("ANALISI_GB300_FAIL_ALLOC");
    if (e && (std::strcmp(e, "1") == 0 || (tag && std::strcmp(e, tag) == 0))) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(reinterpret_cast<void **>(p), bytes);
}

struct DevGuard {
    int prev = -1;
    explicit DevGuard(int d)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != d) cudaSetDevice(d);
    }
    ~DevGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

template <typename T>
int ensure(gofr_ctx *ctx, T *&p, size_t &cap, size_t n)
{
    if (n <= cap && p) return GOFR_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    CK(dev_malloc(&p, bytes));
    cap = n;
    return GOFR_OK;
}

void free_traj(TrajDev &t)
{
    cudaFree(t.pos64);
    cudaFree(t.pos32);
    cudaFree(t.box64);
    cudaFree(t.box32);
    cudaFree(t.types);
    cudaFree(t.types8);
    cudaFree(t.d_cstart);
    cudaFree(t.d_sidt);
    cudaFree(t.d_spos);
    cudaFree(t.d_wpos);
    t.d_wpos = nullptr;
    cudaFree(t.d_perm);
    cudaFree(t.d_tbegin);
    cudaFree(t.d_cm);
    t.d_perm = nullptr; t.d_tbegin = nullptr; t.d_cm = nullptr;
    t.pos64 = nullptr; t.pos32 = nullptr; t.box64 = nullptr; t.box32 = nullptr; t.types = nullptr;
    t.types8 = nullptr;
    t.d_cstart = nullptr; t.d_sidt = nullptr; t.d_spos = nullptr;
    t.cell_nc[0] = t.cell_nc[1] = t.cell_nc[2] = 0;
}

inline uint64_t dbits(double x) { uint64_t u; std::memcpy(&u, &x, 8); return u; }
inline double bitsd(uint64_t u) { double x; std::memcpy(&x, &u, 8); return x; }

// Smallest float >= x / largest float <= x / largest float < x.
inline float f_up(double x)
{
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, INFINITY);
    return f;
}
inline float f_down(double x)
{
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -INFINITY);
    return f;
}
inline float f_below(double x)
{
    float f = f_down(x);
    if ((double)f >= x) f = std::nextafter(f, -INFINITY);
    return f;
}

// ---------------------------------------------------------------------------
// Reference binning on the host (lib/src/gofrt.cpp:104,114-118).  Compiled
// without FMA contraction (the build passes -fmad=false / -ffp-contract=off);
// the expressions below contain no multiply-add anyway.
// ---------------------------------------------------------------------------
struct BinMap {
    double rmin, rmax, dr, rmin2, rmax2;
    unsigned nbin;
    explicit BinMap(double rmin_, double rmax_, unsigned nbin_)
        : rmin(rmin_), rmax(rmax_), nbin(nbin_)
    {
        dr = (rmax - rmin) / nbin;
        rmax2 = rmax * rmax;
        rmin2 = rmin * rmin;
    }
    // floorf((float)((sqrt(d2)-rmin)/dr)) as a float: monotone non-decreasing in d2 >= 0
    float raw(double d2) const
    {
        double d = std::sqrt(d2);
        return std::floor((float)((d - rmin) / dr));
    }
};

// smallest non-negative double in [lo, hi] with pred true (pred monotone
// false..true over the ordered doubles), or hi+ when none.
template <typename P>
double first_true(double lo, double hi, P pred)
{
    uint64_t a = dbits(lo), b = dbits(hi);
    if (!pred(hi)) return std::nextafter(hi, INFINITY);
    while (a < b) {
        uint64_t m = a + (b - a) / 2;
        if (pred(bitsd(m))) b = m;
        else a = m + 1;
    }
    return bitsd(a);
}

bool regular_bins(double rmin, double rmax, unsigned nbin)
{
    if (!std::isfinite(rmin) || !std::isfinite(rmax) || !(rmax > rmin) || nbin == 0) return false;
    if (nbin >= (1u << 24)) return false;
    double dr = (rmax - rmin) / nbin;
    if (!(dr > 0.0) || !std::isfinite(dr)) return false;
    if (!std::isfinite(rmax * rmax) || !std::isfinite(rmin * rmin)) return false;
    return true;
}

// th[0..nbin]; returns false when the accepted window is empty.
bool thresholds(const BinMap &bm, double *th)
{
    const double top = bitsd(0x7FEFFFFFFFFFFFFFull);
    double P = first_true(0.0, top, [&](double x) { return bm.raw(x) >= 0.0f; });
    double Q = first_true(0.0, top, [&](double x) { return bm.raw(x) >= (float)bm.nbin; });
    double A = std::max(bm.rmin2, P);
    double B = std::min(bm.rmax2, std::nextafter(Q, -INFINITY));
    if (!(A <= B)) {
        for (unsigned b = 0; b <= bm.nbin; ++b) th[b] = 0.0;
        return false;
    }
    th[0] = A;
    double Bp = std::nextafter(B, INFINITY);
    for (unsigned b = 1; b < bm.nbin; ++b)
        th[b] = first_true(A, B, [&](double x) { return bm.raw(x) >= (float)b; });
    for (unsigned b = 1; b < bm.nbin; ++b)
        if (th[b] > Bp) th[b] = Bp;
    th[bm.nbin] = Bp;
    return true;
}

// ---------------------------------------------------------------------------
// Certified FP32 error bound.
//
// The FP32 kernel computes, per axis, d = fl32(a_i - a_j) from coordinates
// a = fl32(fl64(x - shift)), wraps it with k = rint(d/L) and an FMA
// d - k*fl32(L) (triclinic: the z and y wraps also subtract k*fl32(tilt)),
// and forms d2 = fma(z,z, fma(y,y, x*x)).  For every pair whose wrap counts k
// equal the reference's, each final component differs from the reference's
// by at most e_k + 2^-24 |x_k|, where e_k collects (all bounds are maxima
// over frames):
//   2 eps_k                 quantisation of both coordinates, eps = 2^-24 M
//   2^-24 (D_k + 2 eps_k)   rounding of the FP32 difference, D = 2 M
//   2^-53 D_k               rounding of the reference's FP64 difference
//   k_max (|fl32(L)-L| + 2^-53 (D+L))    FP32 box edge, reference's k roundings
//   (triclinic) the same for the tilt terms, plus 2^-24 of each intermediate.
// Summing squares with Cauchy-Schwarz gives, with e = ||e_k||_2 and s the
// reference d2:
//   |d2_f32 - d2_ref| <= E(s) = (2 sqrt(s) e + 2 e^2 + 5.01 * 2^-24 s) (1 + 2^-20)
// (the last term covers 2^-23 s from the relative component error, three FP32
// roundings of the sum and four FP64 roundings of the reference).  E and
// s - E(s) are both increasing in s, which is what the window construction
// in certify() uses.
// ---------------------------------------------------------------------------
struct Bound {
    double e[3];       // per-axis absolute component error
    double enorm;      // ||e||_2
    double eta;        // max error of a wrap quotient d/L (for the wrap check)
    double kmax[3];
};

Bound error_bound(const TrajDev &t)
{
    Bound b{};
    const double u24 = std::ldexp(1.0, -24), u53 = std::ldexp(1.0, -53);
    double eps[3], D[3], eraw[3];
    for (int k = 0; k < 3; ++k) {
        eps[k] = t.M[k] * u24 * (1.0 + std::ldexp(1.0, -20)) + t.M[k] * std::ldexp(1.0, -52);
        D[k] = 2.0 * t.M[k] * (1.0 + std::ldexp(1.0, -40)) + 2.0 * eps[k];
        eraw[k] = 2.0 * eps[k] + u24 * (D[k] + 2.0 * eps[k]) + u53 * D[k];
    }
    const BoxStats &s = t.bs;
    auto kmax_of = [](double Dk, double Lmin) { return std::floor(Dk / Lmin + 0.5) + 1.0; };
    if (!t.tric) {
        for (int k = 0; k < 3; ++k) {
            b.kmax[k] = kmax_of(D[k], s.Lmin[k]);
            b.e[k] = eraw[k] + b.kmax[k] * (s.eL[k] + u53 * (D[k] + s.Lmax[k]));
        }
    } else {
        // z
        b.kmax[2] = kmax_of(D[2], s.Lmin[2]);
        b.e[2] = eraw[2] + b.kmax[2] * (s.eL[2] + u53 * (D[2] + s.Lmax[2]));
        // y after the z wrap (tilt yz = tilt index 2)
        double Dy = D[1] + b.kmax[2] * s.tmax[2];
        double ey1 = eraw[1] + b.kmax[2] * (s.eT[2] + u53 * Dy) + u24 * Dy;
        b.kmax[1] = kmax_of(Dy, s.Lmin[1]);
        b.e[1] = ey1 + b.kmax[1] * (s.eL[1] + u53 * (Dy + s.Lmax[1]));
        // x after the z (xz = tilt 1) and y (xy = tilt 0) wraps
        double Dx = D[0] + b.kmax[2] * s.tmax[1] + b.kmax[1] * s.tmax[0];
        double ex2 = eraw[0] + b.kmax[2] * (s.eT[1] + u53 * Dx) + u24 * Dx +
                     b.kmax[1] * (s.eT[0] + u53 * Dx) + u24 * Dx;
        b.kmax[0] = kmax_of(Dx, s.Lmin[0]);
        b.e[0] = ex2 + b.kmax[0] * (s.eL[0] + u53 * (Dx + s.Lmax[0]));
        D[1] = Dy;
        D[0] = Dx;
    }
    b.enorm = std::sqrt(b.e[0] * b.e[0] + b.e[1] * b.e[1] + b.e[2] * b.e[2]);
    b.eta = 0.0;
    for (int k = 0; k < 3; ++k) {
        double eq = b.e[k] / s.Lmin[k] + (D[k] / s.Lmin[k] + 1.0) * std::ldexp(1.0, -22);
        b.eta = std::max(b.eta, eq);
    }
    return b;
}

// Per-axis error bound of the cell-list kernel's FP32 differences, for an
// orthorhombic box that is the same in every frame (u = 2^-24, v = 2^-53,
// per axis: xlo, L, L32 = fl32(L), c = fl64(xlo + L/2)).
//   w = fl64(x - n L), n = floor(fl64(fl64(x - xlo) / L)):   |w - (x - nL)| <= v |w|
//     |w - c| <= Mw = L/2 + 3 v (X + L) + v (|xlo| + L), X >= |x - xlo|
//     (fl64 of the quotient may move n by one next to an integer)
//   a = fl32(fl64(w - c)):                   |a - (w - c)| <= (u + 2v) Mw = d3
//   b = fl32(a_j + s L32), s in {-1, 0, 1}:  |b - (a_j + s L32)| <= u (|a| + L32) = d4
//   a_i - b = d*_K + s (L - L32) + (w/a roundings of i and j), K the image
//     n_i - n_j + s, d*_K = x_i - x_j - K L exactly
//   dx = fl32(a_i - b):  |dx - (a_i - b)| <= u |a_i - b| <= u (2 |a| + L32)
// plus the reference's own FP64 rounding of its difference and of kmax wrap
// steps (as in error_bound).  d2 is then formed as in the all-pairs kernel
// (one multiply, two FMAs), so Efun applies with these e.
Bound error_bound_cells(const TrajDev &t)
{
    Bound b{};
    const double u = std::ldexp(1.0, -24), v = std::ldexp(1.0, -53);
    const BoxStats &s = t.bs;
    for (int k = 0; k < 3; ++k) {
        const double L = s.Lmax[k], xlo = t.h_box[k];
        const double c = xlo + 0.5 * L;
        const double X = t.M[k] + std::fabs(t.shift[k] - xlo);
        const double Mw = 0.5 * L + 3.0 * v * (X + L) + v * (std::fabs(xlo) + L);
        const double d1 = v * (std::fabs(c) + Mw);
        const double d3 = (u + 2.0 * v) * Mw;
        const double A = Mw * (1.0 + 2.0 * u) + d3;
        const double L32 = L + s.eL[k];
        const double d4 = u * (A + L32);
        const double ea = s.eL[k] + 2.0 * d1 + 2.0 * d3 + d4;
        const double esub = u * (2.0 * A + L32 + d4);
        const double D = 2.0 * t.M[k] * (1.0 + std::ldexp(1.0, -40));
        const double kmax = std::floor(D / s.Lmin[k] + 0.5) + 1.0;
        const double eref = v * D + kmax * v * (D + s.Lmax[k]);
        b.e[k] = (ea + esub + eref) * (1.0 + std::ldexp(1.0, -20));
        b.kmax[k] = kmax;
    }
    b.enorm = std::sqrt(b.e[0] * b.e[0] + b.e[1] * b.e[1] + b.e[2] * b.e[2]);
    b.eta = 0.0;  // no wrap quotients: the cell path needs no wrap check
    return b;
}

// FP64-level slop of the cell lists, per axis (v = 2^-53; the box is the
// same in every frame; X >= |x - xlo| over the coordinates):
//   eref  the reference's own rounding of its difference and of its wrap
//         steps (triclinic: the tilt steps the z and y wraps add to y and x)
//   ew    rounding of the FP64 reduction w of a coordinate into the cell
//   Mw    bound on |w - c|, c the box centre (a quotient rounding across an
//         integer leaves w just outside [lo, lo + L))
// Triclinic reduction (wrap_tric64): |n_z| <= nz = floor(X_z / Lz) + 2, the
// y input y1 = y - n_z yz has |y1 - ylo| <= Y1 = X_y + nz |yz|, |n_y| <= ny
// likewise, and the x inputs x1 = x - n_z xz, x2 = x1 - n_y xy have
// |x2 - xlo| <= X2 = X_x + nz |xz| + ny |xy|; each FMA rounds once.
struct CellSlop {
    double eref[3], ew[3], Mw[3], kmax[3];
};

CellSlop cell_slop(const TrajDev &t)
{
    CellSlop c{};
    const double v = std::ldexp(1.0, -53), g40 = 1.0 + std::ldexp(1.0, -40);
    const BoxStats &s = t.bs;
    double D[3];
    for (int k = 0; k < 3; ++k) D[k] = 2.0 * t.M[k] * g40;
    auto kmax_of = [](double Dk, double Lmin) { return std::floor(Dk / Lmin + 0.5) + 1.0; };
    if (!t.tric) {
        for (int k = 0; k < 3; ++k) {
            c.kmax[k] = kmax_of(D[k], s.Lmin[k]);
            c.eref[k] = v * D[k] + c.kmax[k] * v * (D[k] + s.Lmax[k]);
        }
    } else {
        c.kmax[2] = kmax_of(D[2], s.Lmin[2]);
        c.eref[2] = v * D[2] + c.kmax[2] * v * (D[2] + s.Lmax[2]);
        const double Dy = D[1] + c.kmax[2] * s.tmax[2];
        c.kmax[1] = kmax_of(Dy, s.Lmin[1]);
        c.eref[1] = v * D[1] + c.kmax[2] * v * Dy + c.kmax[1] * v * (Dy + s.Lmax[1]);
        const double Dx = D[0] + c.kmax[2] * s.tmax[1] + c.kmax[1] * s.tmax[0];
        c.kmax[0] = kmax_of(Dx, s.Lmin[0]);
        c.eref[0] = v * D[0] + (c.kmax[2] + c.kmax[1]) * v * Dx + c.kmax[0] * v * (Dx + s.Lmax[0]);
    }
    double lo[3], L[3], X[3], ctr[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = t.h_box[k];
        L[k] = 2.0 * t.h_box[3 + k];
        X[k] = t.M[k] + std::fabs(t.shift[k] - lo[k]);
        ctr[k] = lo[k] + 0.5 * L[k];
    }
    double Xin[3] = {X[0], X[1], X[2]};  // bound on |input - lo| of each axis's reduction
    double ein[3] = {0.0, 0.0, 0.0};     // rounding of that input
    if (t.tric) {
        const double xy = std::fabs(t.h_box[6]), xz = std::fabs(t.h_box[7]),
                     yz = std::fabs(t.h_box[8]);
        const double nz = std::floor(X[2] / L[2]) + 2.0;
        const double Y1 = (X[1] + nz * yz) * g40;
        const double ny = std::floor(Y1 / L[1]) + 2.0;
        const double X1 = (X[0] + nz * xz) * g40;
        const double X2 = (X[0] + nz * xz + ny * xy) * g40;
        Xin[1] = Y1;
        Xin[0] = X2;
        ein[1] = v * (std::fabs(lo[1]) + Y1);
        ein[0] = v * (std::fabs(lo[0]) + X1) + v * (std::fabs(lo[0]) + X2);
    }
    for (int k = 0; k < 3; ++k) {
        c.Mw[k] = 0.5 * L[k] + 3.0 * v * (Xin[k] + L[k]) + v * (std::fabs(lo[k]) + L[k]);
        c.ew[k] = ein[k] + v * (std::fabs(ctr[k]) + c.Mw[k]);
    }
    return c;
}

// Neighbourhood geometry of the warp-streamed kernel on one cell grid (the
// tables of CellwLaunch) and the FP32 image vectors with their error.
struct CellwGeom {
    int nz_lo = 0, nz_hi = 0, ny_lo[3] = {0, 0, 0}, ny_hi[3] = {0, 0, 0};
    int nx_lo[15] = {}, nx_hi[15] = {};
    int nz_span = 0, ny_span = 0, nx_span = 0;  // widest layer range, row range, cell range
    float4 shift[CELLW_NSHIFT] = {};
    double S[3] = {0, 0, 0};   // max |FP32 image vector| per axis over the images reached
    double eT[3] = {0, 0, 0};  // max |FP32 image vector - lattice vector| per axis
};

inline int floordiv_h(int a, int n) { return a >= 0 ? a / n : -((n - 1 - a) / n); }

// The rows and cells a warp block must reach: every lattice image of a cell
// that comes within rm of the block on each axis, rm = rmax plus the FP64
// slop (the reference's rounding, the reduction's, the cell assignment's
// quotient), so every pair the reference counts is evaluated.  A cell's
// image under (sx, sy, sz) is shifted by sz (xz, yz, Lz) + sy (xy, Ly, 0) +
// sx (Lx, 0, 0): in cells of edge h, a layer's rows start (sz yz / h_y) cells
// off and a row's cells (sz xz + sy xy) / h_x.  Orthorhombic grids (cell
// edge >= rmax (1 + 1e-6) / reach) give lo = -reach, hi = reach - 1 on every
// axis.  False when an image falls outside the table (sx, sy in -2..2,
// sz in -1..1; orthorhombic: every s in -1..1, the block kernel's bound).
bool cellw_geometry(const TrajDev &t, const gofr_params &p, const int nc[3], CellwGeom &g)
{
    g = CellwGeom{};
    const double v = std::ldexp(1.0, -53);
    const CellSlop cs = cell_slop(t);
    const double erefn =
        std::sqrt(cs.eref[0] * cs.eref[0] + cs.eref[1] * cs.eref[1] + cs.eref[2] * cs.eref[2]);
    double L[3], h[3], rho[3];
    for (int k = 0; k < 3; ++k) {
        L[k] = 2.0 * t.h_box[3 + k];
        h[k] = L[k] / nc[k];
        const double rm = (p.rmax + erefn + 2.0 * cs.ew[k] +
                           8.0 * v * (std::fabs(t.h_box[k]) + 2.0 * L[k])) *
                          (1.0 + std::ldexp(1.0, -40));
        rho[k] = rm / h[k];
    }
    const double xy = t.tric ? t.h_box[6] : 0.0, xz = t.tric ? t.h_box[7] : 0.0,
                 yz = t.tric ? t.h_box[8] : 0.0;
    const double tiny = 1e-12;  // floor of a value next to an integer: take the wider range
    g.nz_lo = (int)std::floor(-rho[2] - tiny);
    g.nz_hi = (int)std::floor(rho[2] + tiny);
    g.nz_span = g.nz_hi - g.nz_lo + 1;
    const int smax = t.tric ? 2 : 1;
    const int sz_lo = floordiv_h(g.nz_lo, nc[2]), sz_hi = floordiv_h(nc[2] + g.nz_hi, nc[2]);
    if (sz_lo < -1 || sz_hi > 1) return false;
    int sx_lo = 0, sx_hi = 0, sy_lo = 0, sy_hi = 0;
    for (int sz = sz_lo; sz <= sz_hi; ++sz) {
        const double oy = sz * yz / h[1];
        const int a = (int)std::floor(-rho[1] - oy - tiny), b = (int)std::floor(rho[1] - oy + tiny);
        g.ny_lo[sz + 1] = a;
        g.ny_hi[sz + 1] = b;
        g.ny_span = std::max(g.ny_span, b - a + 1);
        const int ylo = floordiv_h(a, nc[1]), yhi = floordiv_h(nc[1] + b, nc[1]);
        if (ylo < -smax || yhi > smax) return false;
        sy_lo = std::min(sy_lo, ylo);
        sy_hi = std::max(sy_hi, yhi);
        for (int sy = ylo; sy <= yhi; ++sy) {
            const double ox = (sz * xz + sy * xy) / h[0];
            const int c0 = (int)std::floor(-rho[0] - ox - tiny),
                      c1 = (int)std::floor(rho[0] - ox + tiny);
            const int k = (sz + 1) * 5 + sy + 2;
            g.nx_lo[k] = c0;
            g.nx_hi[k] = c1;
            g.nx_span = std::max(g.nx_span, c1 - c0 + 1);
            const int xlo = floordiv_h(c0, nc[0]), xhi = floordiv_h(nc[0] + c1, nc[0]);
            if (xlo < -smax || xhi > smax) return false;
            sx_lo = std::min(sx_lo, xlo);
            sx_hi = std::max(sx_hi, xhi);
        }
    }
    // image vectors: FP64 sum of exact products (|s| <= 2), rounded to FP32
    for (int sz = -1; sz <= 1; ++sz)
        for (int sy = -2; sy <= 2; ++sy)
            for (int sx = -2; sx <= 2; ++sx) {
                double T[3] = {sx * L[0], sy * L[1], sz * L[2]};
                T[0] = T[0] + sy * xy;
                T[0] = T[0] + sz * xz;
                T[1] = T[1] + sz * yz;
                const double mag[3] = {std::fabs(sx * L[0]) + std::fabs(sy * xy) +
                                           std::fabs(sz * xz),
                                       std::fabs(sy * L[1]) + std::fabs(sz * yz),
                                       std::fabs(sz * L[2])};
                float f[3];
                for (int k = 0; k < 3; ++k) f[k] = (float)T[k];
                g.shift[(sx + 2) + 5 * (sy + 2) + 25 * (sz + 1)] =
                    make_float4(f[0], f[1], f[2], 0.0f);
                if (sx < sx_lo || sx > sx_hi || sy < sy_lo || sy > sy_hi || sz < sz_lo ||
                    sz > sz_hi)
                    continue;
                for (int k = 0; k < 3; ++k) {
                    g.S[k] = std::max(g.S[k], (double)std::fabs(f[k]));
                    g.eT[k] = std::max(g.eT[k], std::fabs((double)f[k] - T[k]) + 2.0 * v * mag[k]);
                }
            }
    return true;
}

// Per-axis error bound of the warp-streamed kernel's FP32 differences in a
// triclinic box (the same in every frame), with the slop of cell_slop and
// the image vectors of g (u = 2^-24):
//   a = fl32(fl64(w - c)):              |a - (w - c)| <= (u + 2v) Mw = d3
//   b = fl32(a_j + sh), sh the FP32 image vector (|sh| <= S, |sh - T| <= eT):
//                                       |b - (a_j + sh)| <= u (A + S) = d4
//   a_i - b = the lattice image d*_K of the reference's difference (K the
//     lattice vector of the two reductions and the image) + the reductions'
//     rounding (ew each) + the conversions (d3 each) + (T - sh) + d4
//   dx = fl32(a_i - b):                 |dx - (a_i - b)| <= u (2 A + S + d4)
// plus the reference's own rounding (eref).  For a pair the reference counts
// its image is d*_K itself (the one lattice translate within half the box on
// every axis), so these are its component errors; d2 is then formed as in
// the all-pairs kernel and Efun applies.
Bound error_bound_cells_tric(const TrajDev &t, const CellwGeom &g)
{
    Bound b{};
    const double u = std::ldexp(1.0, -24), v = std::ldexp(1.0, -53);
    const CellSlop cs = cell_slop(t);
    for (int k = 0; k < 3; ++k) {
        const double d3 = (u + 2.0 * v) * cs.Mw[k];
        const double A = cs.Mw[k] * (1.0 + 2.0 * u) + d3;
        const double d4 = u * (A + g.S[k]);
        const double ea = g.eT[k] + 2.0 * cs.ew[k] + 2.0 * d3 + d4;
        const double esub = u * (2.0 * A + g.S[k] + d4);
        b.e[k] = (ea + esub + cs.eref[k]) * (1.0 + std::ldexp(1.0, -20));
        b.kmax[k] = cs.kmax[k];
    }
    b.enorm = std::sqrt(b.e[0] * b.e[0] + b.e[1] * b.e[1] + b.e[2] * b.e[2]);
    b.eta = 0.0;
    return b;
}

inline double Efun(const Bound &b, double s)
{
    if (s < 0) s = 0;
    double E = (2.0 * std::sqrt(s) * b.enorm + 2.0 * b.enorm * b.enorm +
                5.01 * std::ldexp(1.0, -24) * s) * (1.0 + std::ldexp(1.0, -20));
    // slack for the double arithmetic of the window construction itself
    return E * 1.01 + std::ldexp(1.0, -50) * s + 1e-300;
}

struct Windows {
    std::vector<float2> win;
    float hi_f, lo_f;
    double E_rmax;
};

void certify(const Bound &b, const double *th, unsigned nbin, Windows &w)
{
    w.win.resize(nbin);
    for (unsigned k = 0; k < nbin; ++k) {
        float lo = th[k] <= 0.0 ? -INFINITY : f_up(th[k] + Efun(b, th[k]));
        float hi = f_below(th[k + 1] - Efun(b, th[k + 1]));
        w.win[k] = make_float2(lo, hi);
    }
    w.hi_f = f_up(th[nbin] + Efun(b, th[nbin]));
    w.lo_f = th[0] <= 0.0 ? -INFINITY : f_down(th[0] - Efun(b, th[0]));
    w.E_rmax = Efun(b, th[nbin]);
}

struct RunShape {
    unsigned leff = 0, ntimesteps = 0, skip = 1, every = 1, nch = 0;
    unsigned n_lags = 0, n_orig = 0;
    size_t data_length = 0;
};

int shape_of(gofr_ctx *ctx, const TrajDev &t, const gofr_params &p, RunShape &rs)
{
    if (p.nbin == 0) return fail(ctx, GOFR_ERR_ARG, "nbin must be > 0");
    rs.skip = p.skip ? p.skip : 1;
    rs.every = p.every ? p.every : 1;
    rs.ntimesteps = p.ntimesteps;
    rs.leff = (p.ntimesteps < p.tmax || p.tmax == 0) ? p.ntimesteps : p.tmax;
    rs.nch = t.ntypes * (t.ntypes + 1);
    rs.data_length = (size_t)rs.leff * rs.nch * p.nbin;
    rs.n_lags = (rs.leff + rs.every - 1) / rs.every;
    rs.n_orig = (rs.ntimesteps + rs.skip - 1) / rs.skip;
    if ((unsigned long long)rs.leff + rs.ntimesteps + p.primo > (unsigned long long)t.T + 1)
        return fail(ctx, GOFR_ERR_RANGE,
                    "trajectory is too short for this kind of calculation. Select a different "
                    "starting timestep or lower the size of the average or the lenght of the "
                    "time lag");
    return GOFR_OK;
}

// Coordinate extent of axis k, [mn, mx] over every frame: the centre the
// FP32 copies are taken about and the bound M on |x - shift|.
void set_extent(TrajDev &t, int k, double mn, double mx)
{
    t.shift[k] = 0.5 * mn + 0.5 * mx;
    const double m = std::max(std::fabs(mx - t.shift[k]), std::fabs(t.shift[k] - mn));
    t.M[k] = m * (1.0 + std::ldexp(1.0, -40)) + 1e-300;
}

// The frames' boxes (stride 6 or 9 doubles each, internal format) into
// t.h_box (9 per frame, tilts zero when orthorhombic), their statistics t.bs,
// t.box_constant and the FP32 boxes b32 (nframes of them); the message of
// the first bad value, or "".
std::string read_boxes(TrajDev &t, const double *boxes, size_t nframes, size_t stride,
                       std::vector<Box32> &b32)
{
    char msg[160];
    t.h_box.assign(nframes * 9, 0.0);
    BoxStats &s = t.bs;
    for (int k = 0; k < 3; ++k) {
        s.Lmin[k] = INFINITY; s.Lmax[k] = 0; s.eL[k] = 0; s.tmax[k] = 0; s.eT[k] = 0;
    }
    s.lh_min = INFINITY;
    for (size_t f = 0; f < nframes; ++f) {
        const double *src = boxes + f * stride;
        double *dst = &t.h_box[f * 9];
        for (size_t q = 0; q < stride; ++q) {
            if (!std::isfinite(src[q])) {
                std::snprintf(msg, sizeof msg, "non-finite box value in frame %zu", f);
                return msg;
            }
            dst[q] = src[q];
        }
        Box32 &bb = b32[f];
        std::memset(&bb, 0, sizeof bb);
        for (int k = 0; k < 3; ++k) {
            double lh = dst[3 + k];
            if (!(lh > 0.0)) {
                std::snprintf(msg, sizeof msg,
                              "box half edge %d of frame %zu is not positive (%g)", k, f, lh);
                return msg;
            }
            double L = lh * 2.0;
            s.Lmin[k] = std::min(s.Lmin[k], L);
            s.Lmax[k] = std::max(s.Lmax[k], L);
            s.lh_min = std::min(s.lh_min, lh);
            bb.L[k] = (float)L;
            bb.invL[k] = (float)(1.0 / L);
            s.eL[k] = std::max(s.eL[k], std::fabs((double)bb.L[k] - L));
            double tl = dst[6 + k];
            bb.tilt[k] = (float)tl;
            s.tmax[k] = std::max(s.tmax[k], std::fabs(tl));
            s.eT[k] = std::max(s.eT[k], std::fabs((double)bb.tilt[k] - tl));
        }
    }
    t.box_constant = true;
    for (size_t f = 1; f < nframes && t.box_constant; ++f)
        t.box_constant = std::memcmp(&t.h_box[f * 9], &t.h_box[0], 9 * sizeof(double)) == 0;
    return "";
}

// Upload one trajectory into t (device buffers owned by t).
int upload_traj(gofr_ctx *ctx, TrajDev &t, const double *positions, const double *boxes,
                int box_kind, const int *type_ids, unsigned ntypes, size_t natoms, size_t nframes)
{
    if (!positions || !boxes || !type_ids)
        return fail(ctx, GOFR_ERR_ARG, "null positions, boxes or type ids");
    if (natoms == 0 || nframes == 0) return fail(ctx, GOFR_ERR_ARG, "empty trajectory");
    if (natoms > (size_t)INT32_MAX / 2) return fail(ctx, GOFR_ERR_ARG, "too many atoms");
    if (box_kind != GOFR_BOX_ORTHO && box_kind != GOFR_BOX_TRICLINIC)
        return fail(ctx, GOFR_ERR_ARG, "invalid box kind %d", box_kind);
    if (ntypes == 0 || ntypes > 255) return fail(ctx, GOFR_ERR_ARG, "ntypes must be in 1..255");
    for (size_t a = 0; a < natoms; ++a)
        if (type_ids[a] < 0 || (unsigned)type_ids[a] >= ntypes)
            return fail(ctx, GOFR_ERR_ARG, "type id %d of atom %zu outside 0..%u", type_ids[a], a,
                        ntypes - 1);
    t.T = nframes;
    t.N = natoms;
    t.ntypes = ntypes;
    t.tric = box_kind == GOFR_BOX_TRICLINIC;
    const size_t stride = t.tric ? 9 : 6;
    std::vector<Box32> b32(nframes);
    {
        const std::string msg = read_boxes(t, boxes, nframes, stride, b32);
        if (!msg.empty()) return fail(ctx, GOFR_ERR_ARG, "%s", msg.c_str());
    }
    free_traj(t);
    const size_t n3 = nframes * natoms * 3;
    CK(dev_malloc(&t.pos64, n3 * sizeof(double)));
    const size_t NP = padded_natoms(natoms);
    CK(dev_malloc(&t.pos32, nframes * 3 * NP * sizeof(float)));
    CK(dev_malloc(&t.types8, NP));
    CK(dev_malloc(&t.box64, nframes * 9 * sizeof(double)));
    CK(dev_malloc(&t.box32, nframes * sizeof(Box32)));
    CK(dev_malloc(&t.types, natoms * sizeof(int)));
    CK(cudaMemcpyAsync(t.pos64, positions, n3 * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
    ctx->h2d_bytes += n3 * sizeof(double) + nframes * (9 * sizeof(double) + sizeof(Box32)) +
                      natoms * sizeof(int);
    CK(cudaMemcpyAsync(t.box64, t.h_box.data(), nframes * 9 * sizeof(double),
                       cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(t.box32, b32.data(), nframes * sizeof(Box32), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(t.types, type_ids, natoms * sizeof(int), cudaMemcpyHostToDevice,
                       ctx->stream));
    t.h_types.assign(type_ids, type_ids + natoms);
    // atoms sorted by type (stable), for the per-type sums of the MSD
    t.h_tbegin.assign(ntypes + 1, 0);
    for (size_t a = 0; a < natoms; ++a) t.h_tbegin[type_ids[a] + 1]++;
    for (unsigned k = 0; k < ntypes; ++k) t.h_tbegin[k + 1] += t.h_tbegin[k];
    t.h_perm.resize(natoms);
    {
        std::vector<int> fill(t.h_tbegin.begin(), t.h_tbegin.end() - 1);
        for (size_t a = 0; a < natoms; ++a) t.h_perm[fill[type_ids[a]]++] = (int)a;
    }
    CK(dev_malloc(&t.d_perm, natoms * sizeof(int)));
    CK(dev_malloc(&t.d_tbegin, (ntypes + 1) * sizeof(int)));
    CK(cudaMemcpyAsync(t.d_perm, t.h_perm.data(), natoms * sizeof(int), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(t.d_tbegin, t.h_tbegin.data(), (ntypes + 1) * sizeof(int),
                       cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_nonfinite, 0, sizeof(unsigned), ctx->stream));
    ++ctx->launches;
    if (launch_minmax(t.pos64, nframes * natoms, ctx->d_minmax, ctx->d_nonfinite, ctx->stream))
        return fail(ctx, GOFR_ERR_CUDA, "min/max kernel launch failed: %s",
                    cudaGetErrorString(cudaGetLastError()));
    std::vector<double> mm(256 * 6);
    unsigned nonfinite = 0;
    CK(cudaMemcpyAsync(mm.data(), ctx->d_minmax, mm.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(&nonfinite, ctx->d_nonfinite, sizeof(unsigned), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (nonfinite)
        return fail(ctx, GOFR_ERR_ARG,
                    "%u non-finite coordinates: the reference's minimum image would not "
                    "terminate on them", nonfinite);
    for (int k = 0; k < 3; ++k) {
        double mn = INFINITY, mx = -INFINITY;
        for (int b = 0; b < 256; ++b) {
            mn = std::min(mn, mm[b * 6 + k]);
            mx = std::max(mx, mm[b * 6 + 3 + k]);
        }
        set_extent(t, k, mn, mx);
    }
    ++ctx->launches;
    if (launch_convert(t.pos64, t.types, nframes, natoms, t.shift[0], t.shift[1], t.shift[2],
                       t.pos32, t.types8, ctx->stream))
        return fail(ctx, GOFR_ERR_CUDA, "convert kernel launch failed: %s",
                    cudaGetErrorString(cudaGetLastError()));
    CK(cudaStreamSynchronize(ctx->stream));
    return GOFR_OK;
}

std::vector<unsigned short> channel_table(unsigned ntypes)
{
    // lib/include/gofrt.h:86-104
    std::vector<unsigned short> tab(ntypes * ntypes);
    for (unsigned a = 0; a < ntypes; ++a)
        for (unsigned c = 0; c < ntypes; ++c) {
            unsigned t1 = std::min(a, c), t2 = std::max(a, c);
            tab[a * ntypes + c] =
                (unsigned short)(ntypes * (ntypes + 1) / 2 - (t2 + 1) * (t2 + 2) / 2 + t1);
        }
    return tab;
}

struct Plan {
    int kind = 1;              // 0 = FP32+recheck, 1 = FP64
    bool cells = false;        // FP32 kernel in its cell-list form
    int nc[3] = {0, 0, 0}, blk[3] = {1, 1, 1}, nb[3] = {1, 1, 1};
    int reach = 1, cell_r = 4;   // neighbour reach in cells, first atoms per thread
    double cell_fraction = 1.0;  // neighbourhood cells / all cells
    double cell_time = 1e300;    // modelled time / the all-pairs kernel's
    bool cellw = false;          // the warp-streamed form of the cell-list kernel
    int wblk[3] = {1, 1, 1}, nw[3] = {1, 1, 1}, parts = 1;  // its warp blocks
    int cta_warps = 8, hcopy = 1;  // its CTA size and histogram privatisation depth
    CellwGeom geom;                // its neighbourhood tables and image vectors
    bool wrapcheck = false;
    bool empty = false;        // accepted window empty: nothing can be counted
    Windows w;
    Bound b{};
    std::vector<double> th;
};

// One cell-list configuration: cells of edge >= rmax (1 + 1e-6) / reach, so
// two atoms at minimum-image distance <= rmax are at most `reach` cells apart
// on every axis (periodically); at least 2 reach + 1 cells per axis.  A CTA
// takes a block of bx*by*bz cells with r first atoms per thread.
struct CellCand {
    int reach = 1, r = 4;
    int nc[3] = {0, 0, 0};
    std::array<int, 3> blk{{1, 1, 1}};
    double fraction = 1.0;  // neighbourhood cells / all cells
    double cost = 1e300;    // evaluated first-slot x second-atom pairs / N^2
    double time = 1e300;    // modelled time / the all-pairs kernel's
};

// Cell lists need a box that is the same in every frame (the frames share
// one grid) and one reference thread partition; the block kernel also an
// orthorhombic box (the warp-streamed kernel takes triclinic ones).
bool cell_eligible(const TrajDev &t, const gofr_params &p, bool allow_tric = false)
{
    if ((t.tric && !allow_tric) || !t.box_constant || p.nparts > 1) return false;
    if (!(p.rmax > 0.0)) return false;
    if (t.N >= (1u << 24)) return false;  // sorted slots pack type << 24 | atom id
    // large histograms use the global-memory form of the all-pairs kernel
    return cell_smem_bytes((int)(t.ntypes * (t.ntypes + 1)), (int)p.nbin, (int)t.ntypes) <=
           160 * 1024;
}

bool cell_grid(const TrajDev &t, const gofr_params &p, int reach, int nc[3])
{
    long long ncell = 1;
    for (int k = 0; k < 3; ++k) {
        const double L = 2.0 * t.h_box[3 + k];
        const double n = std::floor(L * reach / (p.rmax * (1.0 + 1e-6)));
        if (!(n >= 2.0 * reach + 1.0) || n > 1024.0) return false;
        nc[k] = (int)n;
        ncell *= nc[k];
    }
    // at most 6 cells per atom (+64): the per-frame cell starts then take no
    // more device memory than the frames' FP64 coordinates
    return ncell <= (1ll << 22) && (double)ncell <= 6.0 * (double)t.N + 64.0;
}

// Every configuration, fastest (modelled) first.  The cost counts, over all
// blocks, the first-atom slots a block pays for (its atoms rounded up to
// whole tiles of 256 r, with room for three standard deviations of density
// fluctuation) times the atoms of its neighbourhood, relative to the N^2
// pairs of the all-pairs kernel.  The time model weighs each evaluated pair
// and each candidate (d <= rmax, binned in the warp flush): measured on the
// 16k- and 131k-atom workloads, a candidate costs ~6.8 pair evaluations in
// the all-pairs kernel and ~6.5 in the cell kernel, whose pairs (no wrap
// arithmetic) cost ~0.62 of an all-pairs evaluation.
std::vector<CellCand> cell_candidates(const TrajDev &t, const gofr_params &p)
{
    std::vector<CellCand> all;
    if (!cell_eligible(t, p)) return all;
    const double vbox = 8.0 * t.h_box[3] * t.h_box[4] * t.h_box[5];
    const double f_all = std::min(1.0, 4.18879020478639 * p.rmax * p.rmax * p.rmax / vbox);
    for (int m = 1; m <= 2; ++m) {
        int nc[3];
        if (!cell_grid(t, p, m, nc)) continue;
        const double ncell = (double)nc[0] * nc[1] * nc[2];
        const double per_cell = (double)t.N / ncell;
        for (int bx = 1; bx <= 5; ++bx)
            for (int by = 1; by <= 5; ++by)
                for (int bz = 1; bz <= 5; ++bz) {
                    // each neighbourhood cell once: b + 2 reach <= nc per axis
                    if (bx + 2 * m > nc[0] || by + 2 * m > nc[1] || bz + 2 * m > nc[2]) continue;
                    const int jy = by + 2 * m, jz = bz + 2 * m;
                    if (2 * jy * jz > cell_max_ranges() || by * bz > cell_max_ranges()) continue;
                    const double atoms = per_cell * bx * by * bz;
                    const double nbhd = (double)(bx + 2 * m) * jy * jz;
                    for (int r = 2; r <= 4; ++r) {
                        const int TI = cell_block_atoms(r);
                        const double slots =
                            std::ceil(std::max(atoms + 3.0 * std::sqrt(atoms), 1.0) / TI) * TI;
                        CellCand c;
                        c.reach = m;
                        c.r = r;
                        for (int k = 0; k < 3; ++k) c.nc[k] = nc[k];
                        c.blk = {{bx, by, bz}};
                        c.fraction = nbhd / ncell;
                        const double blocks = (double)((nc[0] + bx - 1) / bx) *
                                              ((nc[1] + by - 1) / by) * ((nc[2] + bz - 1) / bz);
                        c.cost = blocks * slots * nbhd * per_cell / ((double)t.N * t.N);
                        const double f_cell = std::min(1.0, f_all / std::max(c.fraction, 1e-9));
                        c.time = c.cost * (0.62 + 6.5 * f_cell) / (1.0 + 6.8 * f_all);
                        all.push_back(c);
                    }
                }
    }
    std::stable_sort(all.begin(), all.end(),
                     [](const CellCand &a, const CellCand &b) { return a.time < b.time; });
    return all;
}

void apply_cell(Plan &pl, const CellCand &c)
{
    pl.reach = c.reach;
    pl.cell_r = c.r;
    for (int k = 0; k < 3; ++k) {
        pl.nc[k] = c.nc[k];
        pl.blk[k] = c.blk[k];
        pl.nb[k] = (c.nc[k] + c.blk[k] - 1) / c.blk[k];
    }
    pl.cell_fraction = c.fraction;
    pl.cell_time = c.time;
}

// ANALISI_GB300_CELL_PLAN="reach,r,bx,by,bz" fixes the cell-list
// configuration (for reproducible timings); it must be one the planner
// accepts for the job, else the ranked choice stands.
bool cell_override(const TrajDev &t, const gofr_params &p, CellCand &out)
{
    const char *env = std::getenv("ANALISI_GB300_CELL_PLAN");
    if (!env) return false;
    int v[5];
    if (std::sscanf(env, "%d,%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3], &v[4]) != 5) return false;
    for (const CellCand &c : cell_candidates(t, p))
        if (c.reach == v[0] && c.r == v[1] && c.blk[0] == v[2] && c.blk[1] == v[3] &&
            c.blk[2] == v[4]) {
            out = c;
            return true;
        }
    return false;
}

// Turns an FP32 plan (thresholds set) into the cell-list form of configuration
// c, with the cell kernel's own bound and windows.  False when the minimum
// image of the candidates is not certain without a per-pair wrap test.
bool make_cell_plan(const TrajDev &t, const gofr_params &p, Plan &pl, const CellCand &c,
                    const Bound *bound = nullptr)
{
    if (pl.kind != 0 || pl.th.empty()) return false;
    if (t.tric && !bound) return false;  // the block kernel's bound is orthorhombic
    Plan q = pl;
    apply_cell(q, c);
    q.b = bound ? *bound : error_bound_cells(t);
    certify(q.b, q.th.data(), p.nbin, q.w);
    const double emax = std::max(q.b.e[0], std::max(q.b.e[1], q.b.e[2]));
    const double reach = std::sqrt((double)q.w.hi_f) * (1.0 + std::ldexp(1.0, -20)) +
                         2.0 * emax + 1e-9;
    if (!(t.bs.lh_min > reach)) return false;
    q.cells = true;
    q.wrapcheck = false;
    pl = q;
    return true;
}

bool cell_plan(const TrajDev &t, const gofr_params &p, Plan &pl)
{
    CellCand c;
    if (!cell_override(t, p, c)) {
        const std::vector<CellCand> all = cell_candidates(t, p);
        if (all.empty()) return false;
        c = all.front();
    }
    return make_cell_plan(t, p, pl, c);
}

// One configuration of the warp-streamed cell-list kernel: cells of edge >=
// rmax (1 + 1e-6) / reach, warp blocks of w[0] x w[1] x w[2] cells, r first
// atoms per lane.
struct CellwCand {
    int reach = 1, r = 3;
    int nc[3] = {0, 0, 0};
    std::array<int, 3> w{{1, 1, 1}};
    double fraction = 1.0;  // neighbourhood cells of a warp block / all cells
    double cost = 1e300;    // lane-pair slots evaluated / N^2 (+ per-chunk overhead)
};

// Every configuration, cheapest first.  The cost counts, over all warp
// blocks, the block's first atoms times the record slots of its
// neighbourhood's chunks (rows packed 128 records to a chunk, at most 8
// pieces each, so short rows fill chunks less), plus a fixed overhead per
// chunk streamed (one per batch of 64 first atoms; atoms with room for two
// standard deviations of density fluctuation), relative to N^2.  Triclinic
// neighbourhoods take the widest row and cell ranges of their geometry (one
// more than the orthorhombic 2 reach where a tilt shifts them).
std::vector<CellwCand> cellw_candidates(const TrajDev &t, const gofr_params &p)
{
    std::vector<CellwCand> all;
    if (!cell_eligible(t, p, true)) return all;
    // one CTA of 16 warps per SM or two of 8, or not at all
    const int nch = (int)(t.ntypes * (t.ntypes + 1));
    if (cellw_smem_bytes(nch, (int)p.nbin, (int)t.ntypes, 16, 1) > 220 * 1024 &&
        cellw_smem_bytes(nch, (int)p.nbin, (int)t.ntypes, 8, 1) > 110 * 1024)
        return all;
    for (int m = 1; m <= 3; ++m) {
        int nc[3];
        CellwGeom g;
        if (!cell_grid(t, p, m, nc) || !cellw_geometry(t, p, nc, g)) continue;
        const double ncell = (double)nc[0] * nc[1] * nc[2];
        const double per_cell = (double)t.N / ncell;
        for (int wx = 1; wx <= 4; ++wx)
            for (int wy = 1; wy <= 4; ++wy)
                for (int wz = 1; wz <= 4; ++wz) {
                    if (wx + 2 * m > nc[0] || wy + 2 * m > nc[1] || wz + 2 * m > nc[2]) continue;
                    // a row wraps the box at most once
                    if (wx + g.nx_span > nc[0]) continue;
                    const int nrow = (wy + g.ny_span) * (wz + g.nz_span);
                    if (wy * wz > 16 || nrow > CELLW_MAX_ROWS) continue;
                    const double atoms = per_cell * wx * wy * wz;
                    const double rows = (double)nrow;
                    const double row_atoms = per_cell * (wx + g.nx_span);
                    const double nbhd = rows * row_atoms;
                    const double blocks = (double)((nc[0] + wx - 1) / wx) *
                                          ((nc[1] + wy - 1) / wy) * ((nc[2] + wz - 1) / wz);
                    const double chr = cellw_chunk_records();
                    // a row wrapping the box is two pieces
                    const double pieces_per_row = 1.0 + (double)(wx + g.nx_span) / nc[0];
                    const double per_chunk =
                        std::min(chr, cellw_chunk_pieces() * row_atoms / pieces_per_row);
                    const double chunks = std::ceil(nbhd / per_chunk) + 0.5;
                    const double batches =
                        std::ceil(std::max(atoms + 2.0 * std::sqrt(atoms), 1.0) /
                                  cellw_batch_atoms());
                    // a chunk's fixed work (wait, image moves, padding, the last
                    // flush) is about that of six first atoms against its records
                    CellwCand c;
                    c.reach = m;
                    c.r = 4;
                    for (int k = 0; k < 3; ++k) c.nc[k] = nc[k];
                    c.w = {{wx, wy, wz}};
                    c.fraction = rows * (wx + g.nx_span) / ncell;
                    c.cost = blocks * (atoms + 6.0 * batches) * chunks * chr /
                             ((double)t.N * t.N);
                    all.push_back(c);
                }
    }
    std::stable_sort(all.begin(), all.end(),
                     [](const CellwCand &a, const CellwCand &b) { return a.cost < b.cost; });
    return all;
}

// ANALISI_GB300_CELLW_PLAN="reach,4,wx,wy,wz" (4: the records a lane holds)
// fixes the warp-streamed configuration (reproducible timings); it must be
// one the planner accepts.
bool cellw_choice(const TrajDev &t, const gofr_params &p, CellwCand &out)
{
    const std::vector<CellwCand> all = cellw_candidates(t, p);
    if (all.empty()) return false;
    const char *env = std::getenv("ANALISI_GB300_CELLW_PLAN");
    int v[5];
    if (env && std::sscanf(env, "%d,%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3], &v[4]) == 5)
        for (const CellwCand &c : all)
            if (c.reach == v[0] && c.r == v[1] && c.w[0] == v[2] && c.w[1] == v[3] &&
                c.w[2] == v[4]) {
                out = c;
                return true;
            }
    out = all.front();
    return true;
}

// Turns an FP32 plan into the warp-streamed cell-list form (the block cell
// kernel's certified bound and windows: the same wrapped coordinates and
// image moves).
bool make_cellw_plan(const TrajDev &t, const gofr_params &p, Plan &pl, const CellwCand &c)
{
    CellCand cc;
    cc.reach = c.reach;
    cc.r = c.r;
    for (int k = 0; k < 3; ++k) cc.nc[k] = c.nc[k];
    cc.fraction = c.fraction;
    cc.time = c.cost;
    CellwGeom g;
    if (!cellw_geometry(t, p, c.nc, g)) return false;
    Plan q = pl;
    if (t.tric) {
        const Bound b = error_bound_cells_tric(t, g);
        if (!make_cell_plan(t, p, q, cc, &b)) return false;
    } else if (!make_cell_plan(t, p, q, cc)) {
        return false;
    }
    q.cellw = true;
    q.geom = g;
    for (int k = 0; k < 3; ++k) {
        q.wblk[k] = c.w[k];
        q.nw[k] = (c.nc[k] + c.w[k] - 1) / c.w[k];
    }
    // parts of the warp blocks per (lag, origin): items of fewer than 2^31
    // all-pairs-equivalent pairs (the kernel checks the evaluated ones)
    const double n2 = (double)t.N * (double)t.N;
    q.parts = (int)std::max(1.0, std::ceil(n2 / 2147483648.0));
    q.parts = std::min(q.parts, q.nw[0] * q.nw[1] * q.nw[2]);
    // one CTA of 16 warps per SM where its shared memory fits (measured faster
    // on the 16k-atom workload, within 2 % of two CTAs of 8 on the 131k-atom
    // one), else two CTAs of 8; one histogram copy
    q.cta_warps = cellw_smem_bytes((int)(t.ntypes * (t.ntypes + 1)), (int)p.nbin,
                                   (int)t.ntypes, 16, 1) <= 220 * 1024
                      ? 16
                      : 8;
    q.hcopy = 1;
    pl = q;
    return true;
}

// AUTO takes the cell-list form when its modelled time is below this share of
// the all-pairs kernel's (a margin for the model's error).
constexpr double kCellAutoTime = 0.85;
// ... and the warp-streamed form where the block form is not taken (a
// triclinic box, or a box too small for the block form to pay) when its
// modelled lane work is below this share of the all-pairs kernel's pairs (an
// evaluated pair costs it about twice an all-pairs one).
constexpr double kCellwAuto = 0.4;

int make_plan(gofr_ctx *ctx, const TrajDev &t, const gofr_params &p, Plan &pl,
              bool allow_cells = true)
{
    const int req = p.kernel;
    if (req != GOFR_KERNEL_AUTO && req != GOFR_KERNEL_F32_RECHECK && req != GOFR_KERNEL_F64 &&
        req != GOFR_KERNEL_CELL && req != GOFR_KERNEL_TUNED && req != GOFR_KERNEL_CELL_WARP)
        return fail(ctx, GOFR_ERR_ARG, "unknown kernel %d", req);
    if (req == GOFR_KERNEL_TUNED) {
        gofr_params q = p;
        q.kernel = GOFR_KERNEL_AUTO;
        return make_plan(ctx, t, q, pl, allow_cells);
    }
    const bool reg = regular_bins(p.rmin, p.rmax, p.nbin);
    if (reg) {
        pl.th.resize(p.nbin + 1);
        BinMap bm(p.rmin, p.rmax, p.nbin);
        pl.empty = !thresholds(bm, pl.th.data());
    }
    if (req == GOFR_KERNEL_F64 || (!reg && req == GOFR_KERNEL_AUTO)) {
        pl.kind = 1;
        return GOFR_OK;
    }
    if (!reg)
        return fail(ctx, GOFR_ERR_UNSUPPORTED,
                    "the FP32 kernel needs finite rmin < rmax and nbin < 2^24");
    pl.b = error_bound(t);
    certify(pl.b, pl.th.data(), p.nbin, pl.w);
    const double emax = std::max(pl.b.e[0], std::max(pl.b.e[1], pl.b.e[2]));
    const double reach = std::sqrt((double)pl.w.hi_f) * (1.0 + std::ldexp(1.0, -20)) +
                         2.0 * emax + 1e-9;
    pl.kind = 0;
    pl.wrapcheck = !(t.bs.lh_min > reach);
    if (pl.wrapcheck && !(0.5 - pl.b.eta > 0.25)) {
        if (req == GOFR_KERNEL_AUTO) { pl.kind = 1; return GOFR_OK; }
        return fail(ctx, GOFR_ERR_UNSUPPORTED,
                    "coordinates too far outside the box for a certified FP32 wrap");
    }
    if (allow_cells && (req == GOFR_KERNEL_CELL || req == GOFR_KERNEL_AUTO) && !pl.wrapcheck) {
        Plan c = pl;
        if (cell_plan(t, p, c) && (req == GOFR_KERNEL_CELL || c.cell_time < kCellAutoTime))
            pl = c;
    }
    // the warp-streamed form: on request, and for AUTO wherever the block
    // cell-list form was taken and the warp form is eligible (measured faster
    // on every workload where both run), and elsewhere (triclinic boxes,
    // boxes where the block form does not pay) when its modelled lane work is
    // below kCellwAuto of the all-pairs pairs
    if (allow_cells && !pl.wrapcheck &&
        (req == GOFR_KERNEL_CELL_WARP || req == GOFR_KERNEL_AUTO)) {
        CellwCand c;
        Plan q = pl;
        q.cells = false;
        if (cellw_choice(t, p, c) &&
            (req != GOFR_KERNEL_AUTO || pl.cells || c.cost < kCellwAuto) &&
            make_cellw_plan(t, p, q, c))
            pl = q;
    }
    if (req == GOFR_KERNEL_CELL && !pl.cells)
        return fail(ctx, GOFR_ERR_UNSUPPORTED,
                    "the block cell-list kernel needs an orthorhombic box constant over the "
                    "frames with at least 3 cells of edge >= rmax per axis, and nparts <= 1");
    if (req == GOFR_KERNEL_CELL_WARP && !pl.cells)
        return fail(ctx, GOFR_ERR_UNSUPPORTED,
                    "cell lists need a box constant over the frames with at least 3 cells of "
                    "edge >= rmax per axis (triclinic: tilts that keep every image reached "
                    "within two cells' widths of the box), and nparts <= 1");
    return GOFR_OK;
}

int check_device_error(gofr_ctx *ctx)
{
    unsigned e = 0;
    CK(cudaMemcpyAsync(&e, ctx->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (e)
        return fail(ctx, GOFR_ERR_DEVICE, "kernel reported error word 0x%x (%s%s%s%s%s)", e,
                    (e & ERRW_WAIT_TIMEOUT) ? "bounded wait ran out " : "",
                    (e & ERRW_WRAP_LOOP) ? "minimum-image iteration cap " : "",
                    (e & ERRW_QUEUE) ? "work queue overflow " : "",
                    (e & ERRW_BOUNDS) ? "bounds check failed " : "",
                    (e & ERRW_HIST_OVERFLOW) ? "an item evaluated 2^32 pairs or more (run "
                                               "discarded; use the block cell-list kernel)" : "");
    return GOFR_OK;
}

void set_cellw_geometry(CellwLaunch &C, const CellwGeom &g)
{
    C.nz_lo = g.nz_lo;
    C.nz_hi = g.nz_hi;
    for (int k = 0; k < 3; ++k) { C.ny_lo[k] = g.ny_lo[k]; C.ny_hi[k] = g.ny_hi[k]; }
    for (int k = 0; k < 15; ++k) { C.nx_lo[k] = g.nx_lo[k]; C.nx_hi[k] = g.nx_hi[k]; }
    C.ny_span = g.ny_span;
    for (int k = 0; k < CELLW_NSHIFT; ++k) C.shift[k] = g.shift[k];
}

// Builds (once per grid and frames) the cell-sorted copy of t's frames.  On
// any failure every buffer of the cell lists (kept and temporary) is freed
// and the trajectory is left without cell lists (cell_nc 0), so a retry
// starts clean and nothing leaks.
int ensure_cells(gofr_ctx *ctx, const TrajDev &t, const Plan &pl)
{
    TrajDev &tm = const_cast<TrajDev &>(t);
    const bool aos = pl.cellw;  // the warp-streamed kernel's records, else the SoA frames
    if (t.tric && !aos)
        return fail(ctx, GOFR_ERR_UNSUPPORTED, "the block cell-list kernel is orthorhombic");
    if (tm.cell_nc[0] == pl.nc[0] && tm.cell_nc[1] == pl.nc[1] && tm.cell_nc[2] == pl.nc[2] &&
        (aos ? tm.d_wpos != nullptr : tm.d_spos != nullptr))
        return GOFR_OK;
    auto drop_kept = [&tm]() {
        cudaFree(tm.d_cstart); cudaFree(tm.d_sidt); cudaFree(tm.d_spos); cudaFree(tm.d_wpos);
        tm.d_cstart = nullptr; tm.d_sidt = nullptr; tm.d_spos = nullptr; tm.d_wpos = nullptr;
        tm.cell_nc[0] = tm.cell_nc[1] = tm.cell_nc[2] = 0;
    };
    drop_kept();
    const size_t ncell = (size_t)pl.nc[0] * pl.nc[1] * pl.nc[2];
    const size_t NP = padded_natoms(t.N);
    int *cell_of = nullptr, *rank_of = nullptr, *count = nullptr;
    auto drop_temp = [&]() {
        cudaFree(cell_of); cudaFree(rank_of); cudaFree(count);
        cell_of = rank_of = count = nullptr;
    };
    cudaError_t e = dev_malloc(&tm.d_cstart, t.T * (ncell + 1) * sizeof(int), "cells");
    if (aos) {
        if (e == cudaSuccess) e = dev_malloc(&tm.d_wpos, t.T * NP * sizeof(float4), "cells");
    } else {
        if (e == cudaSuccess) e = dev_malloc(&tm.d_sidt, t.T * NP * sizeof(unsigned), "cells");
        if (e == cudaSuccess) e = dev_malloc(&tm.d_spos, t.T * 3 * NP * sizeof(float), "cells");
    }
    if (e == cudaSuccess) e = dev_malloc(&cell_of, t.T * t.N * sizeof(int), "cells");
    if (e == cudaSuccess) e = dev_malloc(&rank_of, t.T * t.N * sizeof(int), "cells");
    if (e == cudaSuccess) e = dev_malloc(&count, t.T * (ncell + 1) * sizeof(int), "cells");
    if (e != cudaSuccess) {
        drop_temp();
        drop_kept();
        (void)cudaGetLastError();
        return fail(ctx, e == cudaErrorMemoryAllocation ? GOFR_ERR_NOMEM : GOFR_ERR_CUDA,
                    "cell-list allocation failed: %s", cudaGetErrorString(e));
    }
    ctx->launches += 3;
    double centre[3];
    for (int k = 0; k < 3; ++k) centre[k] = t.h_box[k] + t.h_box[3 + k];  // xlo + L/2
    int brc = launch_cell_build(t.pos64, t.types8, t.T, t.N, &t.h_box[0], centre, pl.nc,
                                t.tric != 0, cell_of, rank_of, count, tm.d_cstart, tm.d_spos,
                                tm.d_sidt, ctx->stream);
    if (!brc && aos)
        brc = launch_cell_scatter_w(t.pos64, t.types8, t.T, t.N, &t.h_box[0], centre, pl.nc,
                                    t.tric != 0, cell_of, rank_of, tm.d_cstart, tm.d_wpos,
                                    ctx->stream);
    const cudaError_t se = cudaStreamSynchronize(ctx->stream);
    drop_temp();
    if (brc || se != cudaSuccess) {
        drop_kept();
        return fail(ctx, GOFR_ERR_CUDA, "cell-list build failed: %s",
                    cudaGetErrorString(se != cudaSuccess ? se : cudaGetLastError()));
    }
    for (int k = 0; k < 3; ++k) tm.cell_nc[k] = pl.nc[k];
    return GOFR_OK;
}

// Queue every launch of one trajectory's calculate on the stream; counts is
// a device pointer to data_length*(nparts>1?nparts:1) zeroed counts.
int enqueue_run(gofr_ctx *ctx, const TrajDev &t, const gofr_params &p, const RunShape &rs,
                const Plan &pl, unsigned long long *counts, unsigned long long *pairs_out)
{
    *pairs_out = 0;
    if (pl.empty || rs.n_lags == 0 || rs.n_orig == 0 || t.N == 0) return GOFR_OK;
    std::vector<unsigned short> tab = channel_table(t.ntypes);
    int rc = ensure(ctx, ctx->d_chtab, ctx->cap_chtab, tab.size());
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_chtab, tab.data(), tab.size() * sizeof(unsigned short),
                       cudaMemcpyHostToDevice, ctx->stream));
    if (pl.kind == 0) {
        rc = ensure(ctx, ctx->d_win, ctx->cap_win, pl.w.win.size());
        if (rc) return rc;
        CK(cudaMemcpyAsync(ctx->d_win, pl.w.win.data(), pl.w.win.size() * sizeof(float2),
                           cudaMemcpyHostToDevice, ctx->stream));
    }
    int max_smem = 0;
    CK(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    // a histogram that would not leave room for one CTA (with headroom) per SM
    // goes to global memory: slower atomics, same counts
    const bool ghist = pairs_smem_bytes(pl.kind, (int)rs.nch, (int)p.nbin, (int)t.ntypes) >
                       max_smem - 8192;
    const int smem = pairs_smem_bytes(pl.kind, (int)rs.nch, (int)p.nbin, (int)t.ntypes, ghist);
    if (smem > max_smem)
        return fail(ctx, GOFR_ERR_UNSUPPORTED, "kernel needs %d B of shared memory (max %d)",
                    smem, max_smem);
    PairLaunch L{};
    L.pos32 = t.pos32;
    L.types8 = t.types8;
    L.pos64 = t.pos64;
    L.box64 = t.box64;
    L.box32 = t.box32;
    L.win = ctx->d_win;
    L.chtab = ctx->d_chtab;
    L.err = ctx->d_err;
    L.stats = ctx->d_stats;
    L.N = (int)t.N;
    L.NP = (int)padded_natoms(t.N);
    L.nbin = (int)p.nbin;
    L.nch = (int)rs.nch;
    L.ntypes = (int)t.ntypes;
    L.n_lags = (int)rs.n_lags;
    L.every = (int)rs.every;
    L.n_orig = (int)rs.n_orig;
    L.skip = (int)rs.skip;
    L.primo = (long long)p.primo;
    L.tric = t.tric;
    L.ghist = ghist ? 1 : 0;
#ifdef GOFR_DEBUG_BOUNDS
    {
        // test hook of the debug build: ANALISI_GB300_DEBUG_STALL=1 makes the
        // all-pairs FP32 kernel's first bounded wait run out with no copy in
        // flight; the run must end with GOFR_ERR_DEVICE and a usable context
        const char *st = std::getenv("ANALISI_GB300_DEBUG_STALL");
        L.dbg_stall = (st && std::strcmp(st, "1") == 0) ? 1 : 0;
    }
#endif
    BinMap bm(p.rmin, p.rmax, p.nbin);
    L.rmin = bm.rmin; L.rmax = bm.rmax; L.dr = bm.dr; L.rmin2 = bm.rmin2; L.rmax2 = bm.rmax2;
    if (pl.kind == 0) {
        L.hi_f = pl.w.hi_f;
        L.lo_f = pl.w.lo_f;
        L.rmin_f = (float)p.rmin;
        L.inv_dr_f = (float)(1.0 / bm.dr);
        L.wlim = (float)(0.5 - pl.b.eta);
    }
    if (pl.cells && pl.cellw && !ghist) {
        int brc = ensure_cells(ctx, t, pl);
        if (brc) return brc;
        CellwLaunch C{};
        C.pair = L;
        C.pair.a0 = 0;
        C.pair.a1 = (int)t.N;
        C.pair.counts = counts;
        const int nwb = pl.nw[0] * pl.nw[1] * pl.nw[2];
        // items: (lag, origin, part); at least 8 per SM, so few (lag, origin)
        // pairs still fill the GPU
        const long long lo = (long long)L.n_lags * L.n_orig;
        long long parts = std::max<long long>(pl.parts, (8LL * ctx->num_sms + lo - 1) / lo);
        parts = std::min<long long>(parts, nwb);
        C.parts = (int)std::max<long long>(parts, 1);
        C.pair.n_items = lo * C.parts;
        C.start = t.d_cstart;
        C.wpos = t.d_wpos;
        for (int k = 0; k < 3; ++k) { C.nc[k] = pl.nc[k]; C.w[k] = pl.wblk[k]; C.nw[k] = pl.nw[k]; }
        C.reach = pl.reach;
        C.r = pl.cell_r;
        C.cta_warps = pl.cta_warps;
        C.hcopy = pl.hcopy;
        set_cellw_geometry(C, pl.geom);
        if (cellw_smem_bytes(L.nch, L.nbin, L.ntypes, C.cta_warps, C.hcopy) > max_smem)
            return fail(ctx, GOFR_ERR_UNSUPPORTED, "cell-list histogram does not fit shared memory");
        ++ctx->launches;
        if (launch_cellw_pairs(C, ctx->num_sms, ctx->stream))
            return fail(ctx, GOFR_ERR_CUDA, "warp-streamed cell pair kernel launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
        *pairs_out = (unsigned long long)rs.n_lags * rs.n_orig * t.N * t.N;
        return GOFR_OK;
    }
    if (pl.cells && !ghist) {
        int brc = ensure_cells(ctx, t, pl);
        if (brc) return brc;
        CellLaunch C{};
        C.pair = L;
        C.pair.a0 = 0;
        C.pair.a1 = (int)t.N;
        C.pair.counts = counts;
        C.pair.n_items = (long long)L.n_lags * pl.nb[0] * pl.nb[1] * pl.nb[2] * L.n_orig;
        C.start = t.d_cstart;
        C.spos = t.d_spos;
        C.sidt = t.d_sidt;
        for (int k = 0; k < 3; ++k) { C.nc[k] = pl.nc[k]; C.b[k] = pl.blk[k]; C.nb[k] = pl.nb[k]; }
        C.reach = pl.reach;
        C.r = pl.cell_r;
        const int csmem = cell_smem_bytes(L.nch, L.nbin, L.ntypes);
        if (csmem > max_smem)
            return fail(ctx, GOFR_ERR_UNSUPPORTED, "cell-list histogram does not fit shared memory");
        ++ctx->launches;
        if (launch_cell_pairs(C, ctx->num_sms, ctx->stream))
            return fail(ctx, GOFR_ERR_CUDA, "cell pair kernel launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
        *pairs_out = (unsigned long long)rs.n_lags * rs.n_orig * t.N * t.N;
        return GOFR_OK;
    }
    const unsigned nparts = p.nparts > 1 ? p.nparts : 1;
    const int TI = pairs_tile_atoms(pl.kind);
    const size_t per = t.N / nparts;
    for (unsigned q = 0; q < nparts; ++q) {
        size_t a0 = q * per, a1 = (q == nparts - 1) ? t.N : (q + 1) * per;
        if (a1 <= a0) continue;
        L.a0 = (int)a0;
        L.a1 = (int)a1;
        L.n_itiles = (int)((a1 - a0 + TI - 1) / TI);
        L.n_items = (long long)L.n_lags * L.n_itiles * L.n_orig;
        L.counts = counts + (size_t)q * rs.data_length;
        ++ctx->launches;
        if (launch_pairs(L, pl.kind, pl.wrapcheck, ctx->num_sms, ctx->stream, nullptr))
            return fail(ctx, GOFR_ERR_CUDA, "pair kernel launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
    }
    *pairs_out = (unsigned long long)rs.n_lags * rs.n_orig * t.N * t.N;
    return GOFR_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: for GOFR_KERNEL_TUNED, times the all-pairs FP32 kernel and the
// cell-list kernel in its best-estimated configurations (reach, atoms per
// thread, block shape) on a sample of the job (its first origin and first
// lags) and keeps the fastest per key.
// ---------------------------------------------------------------------------
struct TuneChoice {
    int kind = 0;               // 0 all pairs, 1 block cell lists, 2 warp-streamed cell lists
    int reach = 1, r = 4;
    std::array<int, 3> blk{{1, 1, 1}};  // cells per block (1) or per warp block (2)
    int cta_warps = 8, hcopy = 1;       // warp-streamed form: CTA size, histogram copies
};

std::mutex g_tune_mutex;
std::map<std::string, TuneChoice> g_tune;
bool g_tune_loaded = false;

std::string tune_key(const TrajDev &t, const gofr_params &p)
{
    int lg = 0;
    while ((1ull << (lg + 1)) <= (unsigned long long)t.N) ++lg;
    std::ostringstream k;
    k << "n2^" << lg << "_bins" << p.nbin << "_types" << t.ntypes << (t.tric ? "_tric" : "_ortho");
    int nc[3];
    if (cell_eligible(t, p, true) && cell_grid(t, p, 2, nc))
        k << "_halfcells" << nc[0] << "x" << nc[1] << "x" << nc[2];
    else if (cell_eligible(t, p, true) && cell_grid(t, p, 1, nc))
        k << "_cells" << nc[0] << "x" << nc[1] << "x" << nc[2];
    return k.str();
}

// Cache file lines: key kind reach r b0 b1 b2 cta_warps hcopy (lines of an
// older form, key cells reach r b0 b1 b2, are read as kinds 0/1; other lines
// are skipped).
void tune_load_file()
{
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = std::getenv("ANALISI_GB300_TUNE_CACHE");
    if (!path) return;
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string key;
        int kind, m, r, b0, b1, b2;
        if (!(ls >> key >> kind >> m >> r >> b0 >> b1 >> b2)) continue;
        TuneChoice c;
        c.kind = kind;
        c.reach = m;
        c.r = r;
        c.blk = {{b0, b1, b2}};
        int cw, hc;
        if (ls >> cw >> hc) {
            c.cta_warps = cw;
            c.hcopy = hc;
        }
        if (c.kind < 0 || c.kind > 2) continue;
        g_tune[key] = c;
    }
}

void tune_store_file(const std::string &key, const TuneChoice &c)
{
    const char *path = std::getenv("ANALISI_GB300_TUNE_CACHE");
    if (!path) return;
    std::ofstream out(path, std::ios::app);
    out << key << " " << c.kind << " " << c.reach << " " << c.r << " " << c.blk[0] << " "
        << c.blk[1] << " " << c.blk[2] << " " << c.cta_warps << " " << c.hcopy << "\n";
}

// ANALISI_GB300_TUNE_LOG=path appends each timed configuration of the tuner.
void tune_log(const std::string &key, const TuneChoice &c, double ms)
{
    const char *path = std::getenv("ANALISI_GB300_TUNE_LOG");
    if (!path) return;
    std::ofstream out(path, std::ios::app);
    static const char *names[3] = {"all-pairs", "block-cells", "warp-cells"};
    out << key << " " << names[c.kind];
    if (c.kind)
        out << " reach=" << c.reach << " r=" << c.r << " blk=" << c.blk[0] << "x" << c.blk[1]
            << "x" << c.blk[2];
    if (c.kind == 2) out << " cta_warps=" << c.cta_warps << " hcopy=" << c.hcopy;
    out << " ms=" << ms << "\n";
}

int enqueue_run(gofr_ctx *ctx, const TrajDev &t, const gofr_params &p, const RunShape &rs,
                const Plan &pl, unsigned long long *counts, unsigned long long *pairs_out);

// Times one plan on the sample parameters; returns milliseconds (or < 0).
double tune_time(gofr_ctx *ctx, const TrajDev &t, const gofr_params &q, const Plan &pl)
{
    RunShape rs;
    if (shape_of(ctx, t, q, rs)) return -1.0;
    if (ensure(ctx, ctx->d_counts, ctx->cap_counts, rs.data_length)) return -1.0;
    double best = -1.0;
    for (int rep = 0; rep < 2; ++rep) {  // the first run also builds cell lists
        if (cudaMemsetAsync(ctx->d_counts, 0, rs.data_length * 8, ctx->stream) != cudaSuccess)
            return -1.0;
        cudaEventRecord(ctx->ev[1], ctx->stream);
        unsigned long long pairs = 0;
        if (enqueue_run(ctx, t, q, rs, pl, ctx->d_counts, &pairs)) {
            ctx->err.clear();
            (void)cudaGetLastError();
            return -1.0;
        }
        cudaEventRecord(ctx->ev[2], ctx->stream);
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return -1.0;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
        best = ms;
    }
    return best;
}

// The plan of a tuned choice, built on the all-pairs plan base.
bool plan_of_choice(const TrajDev &t, const gofr_params &p, const Plan &base, const TuneChoice &c,
                    Plan &out)
{
    out = base;
    out.cells = false;
    out.cellw = false;
    if (c.kind == 0) return true;
    if (c.kind == 1) {
        for (const CellCand &cc : cell_candidates(t, p))
            if (cc.reach == c.reach && cc.r == c.r && cc.blk == c.blk) {
                Plan q = base;
                if (!make_cell_plan(t, p, q, cc)) return false;
                out = q;
                return true;
            }
        return false;
    }
    for (const CellwCand &cw : cellw_candidates(t, p))
        if (cw.reach == c.reach && cw.r == c.r && cw.w == c.blk) {
            Plan q = base;
            q.cells = false;
            if (!make_cellw_plan(t, p, q, cw)) return false;
            q.cta_warps = c.cta_warps;
            q.hcopy = c.hcopy;
            out = q;
            return true;
        }
    return false;
}

// True when the tuner has a choice for this job's key (in this process, or in
// the file that ANALISI_GB300_TUNE_CACHE names).
bool tune_known(const TrajDev &t, const gofr_params &p)
{
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    tune_load_file();
    return g_tune.count(tune_key(t, p)) != 0;
}

// Applies the tuned choice for p to the all-pairs plan pl, measuring the
// candidates first when the key has no choice yet: the all-pairs kernel, the
// block cell-list kernel in its best modelled configurations, and the
// warp-streamed cell-list kernel in its best modelled configurations, each
// with CTAs of 8 and 16 warps and one or two copies of the shared histogram.
int tune_plan(gofr_ctx *ctx, const TrajDev &t, const gofr_params &p, Plan &pl)
{
    if (pl.kind != 0 || pl.wrapcheck || pl.empty) return GOFR_OK;  // nothing to choose
    const std::string key = tune_key(t, p);
    const Plan base_pl = pl;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        tune_load_file();
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            Plan q;
            if (plan_of_choice(t, p, base_pl, it->second, q)) pl = q;
            return GOFR_OK;
        }
    }
    const std::vector<CellCand> all = cell_candidates(t, p);
    const std::vector<CellwCand> allw = cellw_candidates(t, p);
    if (all.empty() && allw.empty()) {
        pl.cells = false;
        return GOFR_OK;
    }
    // sample of the job: its first origins and first lags, about eight
    // (lag, origin) items per SM (as many as a long job keeps in flight, so
    // no kernel is timed on items split finer than the job's) and at most
    // 3e11 ordered pairs
    const unsigned leff = (p.ntimesteps < p.tmax || p.tmax == 0) ? p.ntimesteps : p.tmax;
    const unsigned skip = p.skip ? p.skip : 1;
    const double n2 = (double)t.N * (double)t.N;
    const double items = std::max(16.0, std::min(8.0 * ctx->num_sms, std::floor(3e11 / n2)));
    const unsigned n_l = (unsigned)std::max<double>(
        1.0, std::min<double>(leff, std::max(4.0, std::ceil(std::sqrt(items)))));
    const unsigned n_o = (unsigned)std::ceil(items / n_l);
    gofr_params q = p;
    q.kernel = GOFR_KERNEL_AUTO;
    q.nparts = 1;
    q.every = 1;
    q.tmax = n_l;
    q.ntimesteps = std::min<unsigned>(p.ntimesteps, std::max<unsigned>(n_l, n_o * skip));
    std::vector<TuneChoice> tries;
    tries.push_back(TuneChoice{});  // all pairs
    // block cell lists: the four cheapest estimates, and the cheapest of each reach
    std::vector<const CellCand *> bc;
    for (size_t c = 0; c < all.size() && bc.size() < 4; ++c) bc.push_back(&all[c]);
    for (int m = 1; m <= 2; ++m)
        for (const CellCand &c : all)
            if (c.reach == m) {
                if (std::find(bc.begin(), bc.end(), &c) == bc.end()) bc.push_back(&c);
                break;
            }
    for (const CellCand *c : bc) {
        TuneChoice tc;
        tc.kind = 1;
        tc.reach = c->reach;
        tc.r = c->r;
        tc.blk = c->blk;
        tries.push_back(tc);
    }
    // warp-streamed: the three cheapest estimates x CTA size x histogram copies
    int max_smem = 0;
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    const int nch = (int)(t.ntypes * (t.ntypes + 1));
    for (size_t c = 0; c < allw.size() && c < 3; ++c)
        for (int cw : {8, 16})
            for (int hc : {1, 2}) {
                if (cellw_smem_bytes(nch, (int)p.nbin, (int)t.ntypes, cw, hc) > max_smem) continue;
                TuneChoice tc;
                tc.kind = 2;
                tc.reach = allw[c].reach;
                tc.r = allw[c].r;
                tc.blk = allw[c].w;
                tc.cta_warps = cw;
                tc.hcopy = hc;
                tries.push_back(tc);
            }
    TuneChoice choice;
    double best_ms = -1.0;
    for (const TuneChoice &tc : tries) {
        Plan cp;
        if (!plan_of_choice(t, p, base_pl, tc, cp)) continue;
        const double ms = tune_time(ctx, t, q, cp);
        tune_log(key, tc, ms);
        if (ms > 0 && (best_ms < 0 || ms < best_ms)) {
            best_ms = ms;
            choice = tc;
        }
    }
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune[key] = choice;
        tune_store_file(key, choice);
    }
    Plan chosen;
    if (plan_of_choice(t, p, base_pl, choice, chosen)) pl = chosen;
    return GOFR_OK;
}

int run_common(gofr_ctx *ctx, const gofr_params *p, unsigned long long *counts_dev,
               unsigned long long *counts_host)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!p) return fail(ctx, GOFR_ERR_ARG, "null params");
    if (ctx->trajs.size() != 1) return fail(ctx, GOFR_ERR_STATE, "no frames uploaded");
    const TrajDev &t = ctx->trajs[0];
    RunShape rs;
    int rc = shape_of(ctx, t, *p, rs);
    if (rc) return rc;
    Plan pl;
    // the tuner starts from the all-pairs plan and decides on cells itself;
    // AUTO takes the tuner's choice when it has one for this job's key
    const bool tuned = p->nparts <= 1 &&
                       (p->kernel == GOFR_KERNEL_TUNED ||
                        (p->kernel == GOFR_KERNEL_AUTO && tune_known(t, *p)));
    rc = make_plan(ctx, t, *p, pl, !tuned);
    if (rc) return rc;
    if (tuned) {
        rc = tune_plan(ctx, t, *p, pl);
        if (rc) return rc;
    }
    if (pl.cells && p->kernel != GOFR_KERNEL_CELL && p->kernel != GOFR_KERNEL_CELL_WARP) {
        // a plan the engine chose (AUTO / TUNED) whose cell lists do not fit
        // the device: the all-pairs form gives the same counts
        const int crc = ensure_cells(ctx, t, pl);
        if (crc == GOFR_ERR_NOMEM) {
            ctx->err.clear();
            (void)cudaGetLastError();
            gofr_params q = *p;
            q.kernel = GOFR_KERNEL_AUTO;
            Plan ap;
            rc = make_plan(ctx, t, q, ap, false);
            if (rc) return rc;
            pl = ap;
        } else if (crc) {
            return crc;
        }
    }
    const unsigned nparts = p->nparts > 1 ? p->nparts : 1;
    const size_t n_out = rs.data_length * nparts;
    unsigned long long *out = counts_dev;
    if (!out) {
        rc = ensure(ctx, ctx->d_counts, ctx->cap_counts, n_out);
        if (rc) return rc;
        out = ctx->d_counts;
    }
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_stats, 0, ST_COUNT * sizeof(unsigned long long), ctx->stream));
    if (n_out) CK(cudaMemsetAsync(out, 0, n_out * sizeof(unsigned long long), ctx->stream));
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    unsigned long long pairs = 0;
    rc = enqueue_run(ctx, t, *p, rs, pl, out, &pairs);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    if (counts_host && n_out)
        CK(cudaMemcpyAsync(counts_host, out, n_out * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    std::memset(&ctx->stats, 0, sizeof ctx->stats);
    ctx->stats.pairs = pairs;
    ctx->stats.evaluated = pairs;
    ctx->stats.kernel_used = pl.kind == 0 ? (pl.cells ? (pl.cellw ? GOFR_KERNEL_CELL_WARP
                                                                  : GOFR_KERNEL_CELL)
                                                      : GOFR_KERNEL_F32_RECHECK)
                                          : GOFR_KERNEL_F64;
    ctx->stats.wrap_checked = pl.wrapcheck ? 1 : 0;
    ctx->stats.err_bound_d2 = pl.kind == 0 ? pl.w.E_rmax : 0.0;
    if (counts_host) return gofr_sync(ctx);
    return GOFR_OK;
}

void free_batch(gofr_ctx *ctx)
{
    auto &B = ctx->batch;
    if (B.graph) cudaGraphExecDestroy(B.graph);
    cudaFree(B.d_launches);
    cudaFree(B.d_work[0]);
    cudaFree(B.d_work[1]);
    cudaFree(B.d_head);
    cudaFree(B.d_win);
    cudaFree(B.d_chtab);
    cudaFree(B.d_counts);
    cudaFree(B.d_cells);
    cudaFree(B.d_cell_end);
    if (B.h_stage) cudaFreeHost(B.h_stage);
    B = gofr_ctx::Batch{};
}

// Plans every trajectory of the batch and lays out the device work queue:
// descriptors of about `target` pairs (never more than 2^31, so no u32
// shared-memory bin can overflow before the flush that ends a descriptor),
// sorted by decreasing cost so the persistent CTAs finish together.
int build_batch(gofr_ctx *ctx)
{
    auto &B = ctx->batch;
    const int TI = pairs_tile_atoms(0);
    std::vector<float2> wins;
    std::vector<unsigned short> tabs;
    std::vector<size_t> win_off(ctx->trajs.size(), 0), tab_off(ctx->trajs.size(), 0);
    unsigned long long total = 0;
    std::vector<Plan> plans(ctx->trajs.size());
    std::vector<RunShape> shapes(ctx->trajs.size());
    std::vector<std::vector<CellCand>> cands(ctx->trajs.size());
    std::vector<double> work(ctx->trajs.size(), 0.0);
    for (size_t k = 0; k < ctx->trajs.size(); ++k) {
        TrajDev &t = ctx->trajs[k];
        gofr_params p = t.params;
        p.kernel = GOFR_KERNEL_AUTO;
        p.nparts = 1;
        int rc = shape_of(ctx, t, p, shapes[k]);
        if (rc) return rc;
        rc = make_plan(ctx, t, p, plans[k], false);  // all-pairs plan; cells decided below
        if (rc) return rc;
        const unsigned long long pk = (unsigned long long)shapes[k].n_lags * shapes[k].n_orig * t.N * t.N;
        total += pk;
        work[k] = (double)pk;
        if (plans[k].kind == 0 && !plans[k].wrapcheck && !plans[k].empty)
            cands[k] = cell_candidates(t, p);
    }
    B.pairs = total;
    // One cell-list launch serves every member that gains from cell lists; it
    // has one first-atoms-per-thread count R, the one with the least modelled
    // time over the batch.
    auto best_of = [&](size_t k, int r) -> const CellCand * {
        for (const CellCand &c : cands[k])
            if (c.r == r) return c.time < kCellAutoTime ? &c : nullptr;
        return nullptr;
    };
    {
        double best_total = 1e300;
        for (int r = 2; r <= 4; ++r) {
            double tot = 0.0;
            for (size_t k = 0; k < ctx->trajs.size(); ++k) {
                const CellCand *c = best_of(k, r);
                tot += work[k] * (c ? c->time : 1.0);
            }
            if (tot < best_total) { best_total = tot; B.cell_r = r; }
        }
    }
    std::vector<char> is_cell(ctx->trajs.size(), 0);
    for (size_t k = 0; k < ctx->trajs.size(); ++k) {
        const CellCand *c = best_of(k, B.cell_r);
        gofr_params p = ctx->trajs[k].params;
        p.nparts = 1;
        if (!c) {
            // the warp-streamed form where the block form does not pay, as AUTO
            // takes it for a single trajectory
            CellwCand cw;
            Plan q = plans[k];
            q.cells = false;
            p.kernel = GOFR_KERNEL_AUTO;
            if (plans[k].kind == 0 && !plans[k].wrapcheck && !plans[k].empty &&
                cellw_choice(ctx->trajs[k], p, cw) && cw.cost < kCellwAuto &&
                make_cellw_plan(ctx->trajs[k], p, q, cw)) {
                plans[k] = q;
                is_cell[k] = 1;
            } else {
                B.allpairs_pairs += (unsigned long long)work[k];
            }
            continue;
        }
        Plan q = plans[k];
        if (make_cell_plan(ctx->trajs[k], p, q, *c) &&
            cell_smem_bytes((int)shapes[k].nch, (int)p.nbin, (int)ctx->trajs[k].ntypes) <= 160 * 1024) {
            plans[k] = q;
            is_cell[k] = 1;
        } else {
            B.allpairs_pairs += (unsigned long long)work[k];
        }
    }
    const unsigned long long target =
        std::max<unsigned long long>(total / ((unsigned long long)ctx->num_sms * 2 * 24), 1ull << 24);
    struct Cost { unsigned long long c; WorkDesc w; bool tri; };
    std::vector<Cost> all;
    B.launches.resize(ctx->trajs.size());
    for (size_t k = 0; k < ctx->trajs.size(); ++k) {
        TrajDev &t = ctx->trajs[k];
        const RunShape &rs = shapes[k];
        const Plan &pl = plans[k];
        if (pl.empty || rs.n_lags == 0 || rs.n_orig == 0) continue;
        if (pl.kind != 0) { B.f64_trajs.push_back((int)k); continue; }
        win_off[k] = wins.size();
        wins.insert(wins.end(), pl.w.win.begin(), pl.w.win.end());
        std::vector<unsigned short> tab = channel_table(t.ntypes);
        tab_off[k] = tabs.size();
        tabs.insert(tabs.end(), tab.begin(), tab.end());
        if (is_cell[k]) {
            B.cell_trajs.push_back((int)k);
            B.cell_max_nbin = std::max(B.cell_max_nbin, (int)t.params.nbin);
            B.cell_max_nch = std::max(B.cell_max_nch, (int)rs.nch);
            B.cell_max_ntypes = std::max(B.cell_max_ntypes, (int)t.ntypes);
            continue;
        }
        B.max_nbin = std::max(B.max_nbin, (int)t.params.nbin);
        B.max_nch = std::max(B.max_nch, (int)rs.nch);
        B.max_ntypes = std::max(B.max_ntypes, (int)t.ntypes);
        const int n_itiles = (int)((t.N + TI - 1) / TI);
        for (unsigned l = 0; l < rs.n_lags; ++l)
            for (int it = 0; it < n_itiles; ++it) {
                const unsigned long long tile = std::min<size_t>(TI, t.N - (size_t)it * TI);
                const unsigned long long per_item = tile * t.N;
                unsigned long long chunk = std::max<unsigned long long>(1, target / per_item);
                chunk = std::min<unsigned long long>(chunk, std::max<unsigned long long>(
                                                                1, (1ull << 31) / per_item));
                for (unsigned k0 = 0; k0 < rs.n_orig; k0 += (unsigned)chunk) {
                    const unsigned k1 = (unsigned)std::min<unsigned long long>(k0 + chunk, rs.n_orig);
                    WorkDesc w{(int)k, (int)l, it, (int)k0, (int)k1, 0, 0, 0};
                    all.push_back({(k1 - k0) * per_item, w, t.tric != 0});
                }
            }
    }
    std::stable_sort(all.begin(), all.end(), [](const Cost &a, const Cost &b) { return a.c > b.c; });
    for (auto &c : all) B.work[c.tri ? 1 : 0].push_back(c.w);
    CK(dev_malloc(&B.d_win, std::max<size_t>(wins.size(), 1) * sizeof(float2)));
    CK(dev_malloc(&B.d_chtab, std::max<size_t>(tabs.size(), 1) * sizeof(unsigned short)));
    if (!wins.empty())
        CK(cudaMemcpy(B.d_win, wins.data(), wins.size() * sizeof(float2), cudaMemcpyHostToDevice));
    if (!tabs.empty())
        CK(cudaMemcpy(B.d_chtab, tabs.data(), tabs.size() * sizeof(unsigned short),
                      cudaMemcpyHostToDevice));
    for (size_t k = 0; k < ctx->trajs.size(); ++k) {
        TrajDev &t = ctx->trajs[k];
        const RunShape &rs = shapes[k];
        const Plan &pl = plans[k];
        PairLaunch &L = B.launches[k];
        L = PairLaunch{};
        if (pl.kind != 0 || pl.empty) continue;
        L.pos32 = t.pos32;
        L.types8 = t.types8;
        L.pos64 = t.pos64;
        L.box64 = t.box64;
        L.box32 = t.box32;
        L.win = B.d_win + win_off[k];
        L.chtab = B.d_chtab + tab_off[k];
        L.counts = B.d_counts + t.out_offset;
        L.err = ctx->d_err;
        L.stats = ctx->d_stats;
        L.N = (int)t.N;
        L.NP = (int)padded_natoms(t.N);
        L.nbin = (int)t.params.nbin;
        L.nch = (int)rs.nch;
        L.ntypes = (int)t.ntypes;
        L.a0 = 0;
        L.a1 = (int)t.N;
        L.n_lags = (int)rs.n_lags;
        L.every = (int)rs.every;
        L.n_orig = (int)rs.n_orig;
        L.skip = (int)rs.skip;
        L.primo = (long long)t.params.primo;
        L.n_itiles = (int)((t.N + TI - 1) / TI);
        BinMap bm(t.params.rmin, t.params.rmax, t.params.nbin);
        L.rmin = bm.rmin; L.rmax = bm.rmax; L.dr = bm.dr; L.rmin2 = bm.rmin2; L.rmax2 = bm.rmax2;
        L.hi_f = pl.w.hi_f;
        L.lo_f = pl.w.lo_f;
        L.rmin_f = (float)t.params.rmin;
        L.inv_dr_f = (float)(1.0 / bm.dr);
        L.wlim = (float)(0.5 - pl.b.eta);
        L.tric = t.tric;
        L.wchk = pl.wrapcheck ? 1 : 0;
    }
    // cell-list members: the warp-streamed kernel where it is eligible (one
    // launch per member), else the block kernel (all such members' items back
    // to back in one launch)
    std::vector<int> block_members;
    std::vector<std::pair<unsigned long long, CellwLaunch>> wl;
    for (int k : B.cell_trajs) {
        TrajDev &t = ctx->trajs[k];
        const RunShape &rs = shapes[k];
        gofr_params p = t.params;
        p.kernel = GOFR_KERNEL_AUTO;
        p.nparts = 1;
        CellwCand cw;
        Plan q = plans[k];
        q.cells = false;
        if (!(cellw_choice(t, p, cw) && make_cellw_plan(t, p, q, cw))) {
            if (plans[k].cellw)  // planned for the warp form alone: no block plan to fall back on
                return fail(ctx, GOFR_ERR_UNSUPPORTED, "trajectory %d: warp cell-list plan lost", k);
            block_members.push_back(k);
            continue;
        }
        int rc = ensure_cells(ctx, t, q);
        if (rc) return rc;
        CellwLaunch C{};
        C.pair = B.launches[k];
        C.pair.win = B.d_win + win_off[k];  // the windows of the block plan: same bound
        const long long lo = (long long)rs.n_lags * rs.n_orig;
        const int nwb = q.nw[0] * q.nw[1] * q.nw[2];
        long long parts = std::max<long long>(q.parts, (8LL * ctx->num_sms + lo - 1) / lo);
        C.parts = (int)std::max<long long>(std::min<long long>(parts, nwb), 1);
        C.pair.n_items = lo * C.parts;
        C.start = t.d_cstart;
        C.wpos = t.d_wpos;
        for (int a = 0; a < 3; ++a) { C.nc[a] = q.nc[a]; C.w[a] = q.wblk[a]; C.nw[a] = q.nw[a]; }
        C.reach = q.reach;
        C.r = q.cell_r;
        C.cta_warps = q.cta_warps;  // as a single run of the member
        C.hcopy = 1;
        set_cellw_geometry(C, q.geom);
        wl.push_back({(unsigned long long)work[k], C});
        B.launches[k] = PairLaunch{};  // not in the all-pairs queue
    }
    std::stable_sort(wl.begin(), wl.end(),
                     [](const std::pair<unsigned long long, CellwLaunch> &a,
                        const std::pair<unsigned long long, CellwLaunch> &b) {
                         return a.first > b.first;
                     });
    for (auto &e : wl) B.cellw.push_back(e.second);
    B.cell_trajs = block_members;
    std::vector<long long> cell_end;
    for (int k : B.cell_trajs) {
        TrajDev &t = ctx->trajs[k];
        const Plan &pl = plans[k];
        int rc = ensure_cells(ctx, t, pl);
        if (rc) return rc;
        CellLaunch C{};
        C.pair = B.launches[k];
        C.pair.n_items = (long long)C.pair.n_lags * pl.nb[0] * pl.nb[1] * pl.nb[2] * C.pair.n_orig;
        C.start = t.d_cstart;
        C.spos = t.d_spos;
        C.sidt = t.d_sidt;
        for (int a = 0; a < 3; ++a) { C.nc[a] = pl.nc[a]; C.b[a] = pl.blk[a]; C.nb[a] = pl.nb[a]; }
        C.reach = pl.reach;
        C.r = pl.cell_r;
        B.cells.push_back(C);
        B.cell_items += C.pair.n_items;
        cell_end.push_back(B.cell_items);
        B.launches[k] = PairLaunch{};  // not in the all-pairs queue
    }
    if (!B.cells.empty()) {
        CK(dev_malloc(&B.d_cells, B.cells.size() * sizeof(CellLaunch)));
        CK(dev_malloc(&B.d_cell_end, cell_end.size() * sizeof(long long)));
        CK(cudaMemcpy(B.d_cells, B.cells.data(), B.cells.size() * sizeof(CellLaunch),
                      cudaMemcpyHostToDevice));
        CK(cudaMemcpy(B.d_cell_end, cell_end.data(), cell_end.size() * sizeof(long long),
                      cudaMemcpyHostToDevice));
    }
    CK(dev_malloc(&B.d_launches, std::max<size_t>(B.launches.size(), 1) * sizeof(PairLaunch)));
    CK(cudaMemcpy(B.d_launches, B.launches.data(), B.launches.size() * sizeof(PairLaunch),
                  cudaMemcpyHostToDevice));
    for (int v = 0; v < 2; ++v) {
        if (B.work[v].empty()) continue;
        CK(dev_malloc(&B.d_work[v], B.work[v].size() * sizeof(WorkDesc)));
        CK(cudaMemcpy(B.d_work[v], B.work[v].data(), B.work[v].size() * sizeof(WorkDesc),
                      cudaMemcpyHostToDevice));
    }
    CK(dev_malloc(&B.d_head, 2 * sizeof(unsigned)));
    CK(cudaMallocHost(&B.h_stage, std::max<size_t>(ctx->batch_total, 1) * sizeof(unsigned long long)));
    const int smem = batch_smem_bytes(B.max_nbin, B.max_nch, B.max_ntypes);
    int max_smem = 0;
    CK(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    if (smem > max_smem)
        return fail(ctx, GOFR_ERR_UNSUPPORTED, "batch histograms need %d B of shared memory", smem);
    for (int v = 0; v < 2; ++v) {
        if (B.work[v].empty()) continue;
        if (prepare_batch(B.max_nbin, B.max_nch, B.max_ntypes, v == 1, ctx->num_sms,
                          (int)B.work[v].size(), &B.grid[v]))
            return fail(ctx, GOFR_ERR_CUDA, "batched kernel setup failed");
    }
    if (!B.cells.empty()) {
        const int csmem = cell_smem_bytes(B.cell_max_nch, B.cell_max_nbin, B.cell_max_ntypes);
        if (csmem > max_smem)
            return fail(ctx, GOFR_ERR_UNSUPPORTED, "batch cell-list histograms need %d B", csmem);
        if (prepare_cell_pairs_multi(B.cell_r, B.cell_max_nbin, B.cell_max_nch,
                                     B.cell_max_ntypes, ctx->num_sms, B.cell_items,
                                     &B.cell_grid))
            return fail(ctx, GOFR_ERR_CUDA, "batched cell-list kernel setup failed");
    }
    return GOFR_OK;
}

// The launch sequence of one batch run (captured into a graph or issued directly).
int enqueue_batch(gofr_ctx *ctx)
{
    auto &B = ctx->batch;
    CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_stats, 0, ST_COUNT * sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(B.d_head, 0, 2 * sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(B.d_counts, 0, std::max<size_t>(ctx->batch_total, 1) * 8, ctx->stream));
    if (!B.cellw.empty()) {
        // the warp-streamed members on the second stream, alongside the rest
        CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
        CK(cudaStreamWaitEvent(ctx->stream2, ctx->ev_fork, 0));
        for (const CellwLaunch &C : B.cellw) {
            ++ctx->launches;
            if (launch_cellw_pairs(C, ctx->num_sms, ctx->stream2))
                return fail(ctx, GOFR_ERR_CUDA, "batched warp cell-list launch failed: %s",
                            cudaGetErrorString(cudaGetLastError()));
        }
        CK(cudaEventRecord(ctx->ev_join, ctx->stream2));
    }
    for (int v = 0; v < 2; ++v) {
        if (B.work[v].empty()) continue;
        ++ctx->launches;
        if (launch_batch_grid(B.d_launches, B.d_work[v], (int)B.work[v].size(), B.d_head + v,
                              B.max_nbin, B.max_nch, B.max_ntypes, v == 1, ctx->d_err,
                              ctx->d_stats, B.grid[v], ctx->stream))
            return fail(ctx, GOFR_ERR_CUDA, "batched kernel launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
    }
    if (!B.cells.empty()) {
        ++ctx->launches;
        if (launch_cell_pairs_multi(B.d_cells, B.d_cell_end, (int)B.cells.size(), B.cell_r,
                                    B.cell_max_nbin, B.cell_max_nch, B.cell_max_ntypes,
                                    B.cell_grid, ctx->stream))
            return fail(ctx, GOFR_ERR_CUDA, "batched cell-list kernel launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
    }
    for (int k : B.f64_trajs) {
        TrajDev &t = ctx->trajs[k];
        gofr_params p = t.params;
        p.kernel = GOFR_KERNEL_F64;
        p.nparts = 1;
        RunShape rs;
        int rc = shape_of(ctx, t, p, rs);
        if (rc) return rc;
        Plan pl;
        rc = make_plan(ctx, t, p, pl);
        if (rc) return rc;
        unsigned long long pairs = 0;
        rc = enqueue_run(ctx, t, p, rs, pl, B.d_counts + t.out_offset, &pairs);
        if (rc) return rc;
    }
    if (!B.cellw.empty()) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    CK(cudaMemcpyAsync(B.h_stage, B.d_counts, ctx->batch_total * 8, cudaMemcpyDeviceToHost,
                       ctx->stream));
    return GOFR_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// exported entry points
// ---------------------------------------------------------------------------
extern "C" {

int gofr_ctx_create(gofr_ctx **out, int device)
{
    if (!out) return GOFR_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GOFR_ERR_CUDA;
    if (device < 0 || device >= ndev) return GOFR_ERR_ARG;
    gofr_ctx *ctx = new (std::nothrow) gofr_ctx();
    if (!ctx) return GOFR_ERR_NOMEM;
    ctx->device = device;
    DevGuard g(device);
    int rc = GOFR_OK;
    do {
        if (cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) !=
                cudaSuccess ||
            cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            rc = GOFR_ERR_CUDA;
            break;
        }
        bool ok = true;
        for (auto &e : ctx->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
        ok = ok && cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) == cudaSuccess;
        ok = ok && dev_malloc(&ctx->d_err, sizeof(unsigned)) == cudaSuccess;
        ok = ok && dev_malloc(&ctx->d_stats, ST_COUNT * sizeof(unsigned long long)) == cudaSuccess;
        ok = ok && dev_malloc(&ctx->d_minmax, 256 * 6 * sizeof(double)) == cudaSuccess;
        ok = ok && dev_malloc(&ctx->d_nonfinite, sizeof(unsigned)) == cudaSuccess;
        if (!ok) rc = GOFR_ERR_CUDA;
    } while (0);
    if (rc) {
        gofr_ctx_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return GOFR_OK;
}

void gofr_ctx_destroy(gofr_ctx *ctx)
{
    if (!ctx) return;
    {
        DevGuard g(ctx->device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        for (auto &t : ctx->trajs) free_traj(t);
        free_batch(ctx);
        cudaFree(ctx->d_counts);
        cudaFree(ctx->d_gofr);
        cudaFree(ctx->d_chfac);
        cudaFree(ctx->d_win);
        cudaFree(ctx->d_chtab);
        cudaFree(ctx->d_err);
        cudaFree(ctx->d_stats);
        cudaFree(ctx->d_minmax);
        cudaFree(ctx->d_nonfinite);
        cudaFree(ctx->d_msd_partial);
        cudaFree(ctx->d_msd_out);
        cudaFree(ctx->d_nl_list);
        cudaFree(ctx->d_nl_meta);
        cudaFree(ctx->d_nl_rpos);
        cudaFree(ctx->d_nl_cut2);
        cudaFree(ctx->d_nl_full);

        if (ctx->stream2) cudaStreamSynchronize(ctx->stream2);
        for (auto &e : ctx->ev)
            if (e) cudaEventDestroy(e);
        if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
        if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
        if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
}

const char *gofr_last_error(const gofr_ctx *ctx)
{
    if (!ctx) return "no context (gofr_ctx_create failed or was not called)";
    return ctx->err.c_str();
}

int gofr_set_frames(gofr_ctx *ctx, const double *positions, const double *boxes, int box_kind,
                    const int *type_ids, unsigned ntypes, size_t natoms, size_t nframes)
{
    if (!ctx) return GOFR_ERR_ARG;
    DevGuard g(ctx->device);
    for (auto &t : ctx->trajs) free_traj(t);
    free_batch(ctx);
    ctx->trajs.clear();
    ctx->trajs.emplace_back();
    int rc = upload_traj(ctx, ctx->trajs[0], positions, boxes, box_kind, type_ids, ntypes, natoms,
                         nframes);
    if (rc) {
        free_traj(ctx->trajs[0]);
        ctx->trajs.clear();
    }
    return rc;
}

int gofr_output_size(const gofr_ctx *ctx_c, const gofr_params *p, size_t *n_counts)
{
    gofr_ctx *ctx = const_cast<gofr_ctx *>(ctx_c);
    if (!ctx || !p || !n_counts) return GOFR_ERR_ARG;
    if (ctx->trajs.size() != 1) return fail(ctx, GOFR_ERR_STATE, "no frames uploaded");
    const TrajDev &t = ctx->trajs[0];
    unsigned leff = (p->ntimesteps < p->tmax || p->tmax == 0) ? p->ntimesteps : p->tmax;
    size_t n = (size_t)leff * t.ntypes * (t.ntypes + 1) * p->nbin;
    *n_counts = n * (p->nparts > 1 ? p->nparts : 1);
    return GOFR_OK;
}

int gofr_run(gofr_ctx *ctx, const gofr_params *p, unsigned long long *counts_host)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!counts_host) return fail(ctx, GOFR_ERR_ARG, "null output buffer");
    DevGuard g(ctx->device);
    return run_common(ctx, p, nullptr, counts_host);
}

int gofr_run_device(gofr_ctx *ctx, const gofr_params *p, unsigned long long *counts_device)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!counts_device) return fail(ctx, GOFR_ERR_ARG, "null output buffer");
    DevGuard g(ctx->device);
    return run_common(ctx, p, counts_device, nullptr);
}

}  // extern "C"

namespace {

// Runs the windows; the counts [nwin][nparts][leff][nch][nbin] stay in
// ctx->d_counts and are copied to counts_host when it is not null.
int run_windows_impl(gofr_ctx *ctx, const gofr_params *p, unsigned nwin,
                     const unsigned long long *primos, unsigned long long *counts_host)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!p || !primos || nwin == 0)
        return fail(ctx, GOFR_ERR_ARG, "null argument or no windows");
    if (ctx->trajs.size() != 1) return fail(ctx, GOFR_ERR_STATE, "no frames uploaded");
    DevGuard g(ctx->device);
    const TrajDev &t = ctx->trajs[0];
    const unsigned nparts = p->nparts > 1 ? p->nparts : 1;
    RunShape rs;
    for (unsigned w = 0; w < nwin; ++w) {
        gofr_params q = *p;
        q.primo = primos[w];
        const int rc = shape_of(ctx, t, q, rs);
        if (rc) return rc;
    }
    Plan pl;
    int rc = make_plan(ctx, t, *p, pl);
    if (rc) return rc;
    const size_t per_win = rs.data_length * nparts;
    const size_t n_out = per_win * nwin;
    rc = ensure(ctx, ctx->d_counts, ctx->cap_counts, n_out);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_stats, 0, ST_COUNT * sizeof(unsigned long long), ctx->stream));
    if (n_out) CK(cudaMemsetAsync(ctx->d_counts, 0, n_out * sizeof(unsigned long long), ctx->stream));
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    unsigned long long pairs = 0;
    PairLaunch *d_l = nullptr;
    WorkDesc *d_w = nullptr;
    unsigned *d_head = nullptr;
    int max_smem = 0;
    CK(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    bool one_launch = pl.kind == 0 && !pl.cells && !pl.empty && rs.n_lags > 0 && rs.n_orig > 0 &&
                      batch_smem_bytes((int)p->nbin, (int)rs.nch, (int)t.ntypes) <= max_smem - 8192;
    if (!one_launch) {
        for (unsigned w = 0; w < nwin && rc == GOFR_OK; ++w) {
            gofr_params q = *p;
            q.primo = primos[w];
            unsigned long long pw = 0;
            rc = enqueue_run(ctx, t, q, rs, pl, ctx->d_counts + w * per_win, &pw);
            pairs += pw;
        }
        if (rc) return rc;
    } else {
        // one parameter record per (window, partition), descriptors over all of them
        const int TI = pairs_tile_atoms(0);
        std::vector<unsigned short> tab = channel_table(t.ntypes);
        rc = ensure(ctx, ctx->d_chtab, ctx->cap_chtab, tab.size());
        if (rc == GOFR_OK) rc = ensure(ctx, ctx->d_win, ctx->cap_win, pl.w.win.size());
        if (rc) return rc;
        CK(cudaMemcpyAsync(ctx->d_chtab, tab.data(), tab.size() * sizeof(unsigned short),
                           cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_win, pl.w.win.data(), pl.w.win.size() * sizeof(float2),
                           cudaMemcpyHostToDevice, ctx->stream));
        BinMap bm(p->rmin, p->rmax, p->nbin);
        std::vector<PairLaunch> ls;
        struct Cost { unsigned long long c; WorkDesc w; };
        std::vector<Cost> all;
        const size_t per = t.N / nparts;
        const unsigned long long target = 1ull << 26;
        for (unsigned w = 0; w < nwin; ++w)
            for (unsigned q = 0; q < nparts; ++q) {
                const size_t a0 = q * per, a1 = (q == nparts - 1) ? t.N : (q + 1) * per;
                if (a1 <= a0) continue;
                PairLaunch L{};
                L.pos32 = t.pos32; L.types8 = t.types8; L.pos64 = t.pos64; L.box64 = t.box64;
                L.box32 = t.box32; L.win = ctx->d_win; L.chtab = ctx->d_chtab;
                L.counts = ctx->d_counts + w * per_win + q * rs.data_length;
                L.err = ctx->d_err; L.stats = ctx->d_stats;
                L.N = (int)t.N; L.NP = (int)padded_natoms(t.N);
                L.nbin = (int)p->nbin; L.nch = (int)rs.nch; L.ntypes = (int)t.ntypes;
                L.a0 = (int)a0; L.a1 = (int)a1;
                L.n_lags = (int)rs.n_lags; L.every = (int)rs.every;
                L.n_orig = (int)rs.n_orig; L.skip = (int)rs.skip; L.primo = (long long)primos[w];
                L.n_itiles = (int)((a1 - a0 + TI - 1) / TI);
                L.rmin = bm.rmin; L.rmax = bm.rmax; L.dr = bm.dr; L.rmin2 = bm.rmin2;
                L.rmax2 = bm.rmax2;
                L.hi_f = pl.w.hi_f; L.lo_f = pl.w.lo_f; L.rmin_f = (float)p->rmin;
                L.inv_dr_f = (float)(1.0 / bm.dr); L.wlim = (float)(0.5 - pl.b.eta);
                L.tric = t.tric; L.wchk = pl.wrapcheck ? 1 : 0;
                const int li = (int)ls.size();
                ls.push_back(L);
                for (unsigned l = 0; l < rs.n_lags; ++l)
                    for (int it = 0; it < L.n_itiles; ++it) {
                        const unsigned long long tile =
                            std::min<size_t>(TI, a1 - a0 - (size_t)it * TI);
                        const unsigned long long per_item = tile * t.N;
                        unsigned long long chunk = std::max<unsigned long long>(1, target / per_item);
                        chunk = std::min<unsigned long long>(
                            chunk, std::max<unsigned long long>(1, (1ull << 31) / per_item));
                        for (unsigned k0 = 0; k0 < rs.n_orig; k0 += (unsigned)chunk) {
                            const unsigned k1 =
                                (unsigned)std::min<unsigned long long>(k0 + chunk, rs.n_orig);
                            all.push_back({(k1 - k0) * per_item, WorkDesc{li, (int)l, it, (int)k0,
                                                                       (int)k1, 0, 0, 0}});
                        }
                    }
            }
        std::stable_sort(all.begin(), all.end(),
                         [](const Cost &a, const Cost &b) { return a.c > b.c; });
        std::vector<WorkDesc> work;
        for (auto &c : all) work.push_back(c.w);
        int grid = 0;
        if (prepare_batch((int)p->nbin, (int)rs.nch, (int)t.ntypes, t.tric != 0, ctx->num_sms,
                          (int)work.size(), &grid))
            return fail(ctx, GOFR_ERR_CUDA, "batched kernel setup failed");
        CK(dev_malloc(&d_l, ls.size() * sizeof(PairLaunch)));
        CK(dev_malloc(&d_w, std::max<size_t>(work.size(), 1) * sizeof(WorkDesc)));
        CK(dev_malloc(&d_head, sizeof(unsigned)));
        CK(cudaMemcpyAsync(d_l, ls.data(), ls.size() * sizeof(PairLaunch), cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(cudaMemcpyAsync(d_w, work.data(), work.size() * sizeof(WorkDesc),
                           cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemsetAsync(d_head, 0, sizeof(unsigned), ctx->stream));
        ++ctx->launches;
        if (launch_batch_grid(d_l, d_w, (int)work.size(), d_head, (int)p->nbin, (int)rs.nch,
                              (int)t.ntypes, t.tric != 0, ctx->d_err, ctx->d_stats, grid,
                              ctx->stream))
            rc = fail(ctx, GOFR_ERR_CUDA, "windows launch failed: %s",
                      cudaGetErrorString(cudaGetLastError()));
        pairs = (unsigned long long)nwin * rs.n_lags * rs.n_orig * t.N * t.N;
    }
    if (rc == GOFR_OK) {
        CK(cudaEventRecord(ctx->ev[2], ctx->stream));
        if (n_out && counts_host)
            CK(cudaMemcpyAsync(counts_host, ctx->d_counts, n_out * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaEventRecord(ctx->ev[3], ctx->stream));
        std::memset(&ctx->stats, 0, sizeof ctx->stats);
        ctx->stats.pairs = pairs;
        ctx->stats.evaluated = pairs;
        ctx->stats.kernel_used = pl.kind == 0 ? (pl.cells ? (pl.cellw ? GOFR_KERNEL_CELL_WARP
                                                                      : GOFR_KERNEL_CELL)
                                                          : GOFR_KERNEL_F32_RECHECK)
                                              : GOFR_KERNEL_F64;
        ctx->stats.wrap_checked = pl.wrapcheck ? 1 : 0;
        rc = gofr_sync(ctx);
    }
    cudaStreamSynchronize(ctx->stream);
    cudaFree(d_l);
    cudaFree(d_w);
    cudaFree(d_head);
    return rc;
}

}  // namespace

extern "C" {

int gofr_run_windows(gofr_ctx *ctx, const gofr_params *p, unsigned nwin,
                     const unsigned long long *primos, unsigned long long *counts_host)
{
    if (ctx && !counts_host) return fail(ctx, GOFR_ERR_ARG, "null output buffer");
    return run_windows_impl(ctx, p, nwin, primos, counts_host);
}

int gofr_run_normalized(gofr_ctx *ctx, const gofr_params *p, unsigned nwin,
                      const unsigned long long *primos, int norm, double *out_host,
                      double *rel_err_bound)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!p || !out_host) return fail(ctx, GOFR_ERR_ARG, "null argument");
    if (norm < 0 || norm > 2) return fail(ctx, GOFR_ERR_ARG, "unknown normalisation %d", norm);
    if (ctx->trajs.size() != 1) return fail(ctx, GOFR_ERR_STATE, "no frames uploaded");
    const unsigned long long one = p->primo;
    if (nwin == 0) nwin = 1;
    if (!primos) {
        if (nwin != 1) return fail(ctx, GOFR_ERR_ARG, "several windows need their primos");
        primos = &one;
    }
    DevGuard g(ctx->device);
    int rc = run_windows_impl(ctx, p, nwin, primos, nullptr);
    if (rc) return rc;
    const TrajDev &t = ctx->trajs[0];
    RunShape rs;
    rc = shape_of(ctx, t, *p, rs);
    if (rc) return rc;
    const size_t n = rs.data_length;
    rc = ensure(ctx, ctx->d_gofr, ctx->cap_gofr, std::max<size_t>(n * nwin, 1));
    if (rc) return rc;
    // pair-density factors per channel (mode 2): box volume averaged over the
    // windows' origin frames, atoms per type
    const unsigned nt = t.ntypes, half = nt * (nt + 1) / 2;
    std::vector<double> chfac(2 * half, 1.0);
    if (norm == 2) {
        double vsum = 0.0;
        size_t nv = 0;
        for (unsigned w = 0; w < nwin; ++w)
            for (unsigned k = 0; k < rs.n_orig; ++k) {
                const double *b = &t.h_box[(primos[w] + (size_t)k * rs.skip) * 9];
                vsum += 8.0 * b[3] * b[4] * b[5];
                ++nv;
            }
        const double V = nv ? vsum / nv : 8.0 * t.h_box[3] * t.h_box[4] * t.h_box[5];
        const std::vector<unsigned short> tab = channel_table(nt);
        for (unsigned a = 0; a < nt; ++a)
            for (unsigned c = a; c < nt; ++c) {
                const double na = t.h_tbegin[a + 1] - t.h_tbegin[a];
                const double nc = t.h_tbegin[c + 1] - t.h_tbegin[c];
                const unsigned ch = tab[a * nt + c];
                chfac[ch] = (a == c ? na * (na - 1.0) : 2.0 * na * nc) / V;
                if (a == c) chfac[ch + half] = na;
            }
        rc = ensure(ctx, ctx->d_chfac, ctx->cap_chfac, chfac.size());
        if (rc) return rc;
        CK(cudaMemcpyAsync(ctx->d_chfac, chfac.data(), chfac.size() * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->stream));
    }
    NormLaunch L{};
    L.counts = ctx->d_counts;
    L.out = ctx->d_gofr;
    L.chfac = ctx->d_chfac;
    L.n = n;
    L.nwin = (int)nwin;
    L.nparts = p->nparts > 1 ? (int)p->nparts : 1;
    L.nbin = (int)p->nbin;
    L.nch = (int)rs.nch;
    L.mode = norm;
    L.incr = (rs.ntimesteps / rs.skip > 0) ? 1.0 / (int)(rs.ntimesteps / rs.skip) : 1.0;
    L.r0 = p->rmin;
    L.dr = (p->rmax - p->rmin) / p->nbin;
    L.c43pi = 4.0 * 3.141592653589793 / 3.0;  // numpy: 4 * np.pi / 3
    ++ctx->launches;
    if (launch_counts_to_gofr(L, ctx->num_sms, ctx->stream))
        return fail(ctx, GOFR_ERR_CUDA, "normalisation launch failed: %s",
                    cudaGetErrorString(cudaGetLastError()));
    if (n)
        CK(cudaMemcpyAsync(out_host, ctx->d_gofr, n * nwin * sizeof(double),
                           cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (rel_err_bound) {
        // the cubes here are correctly rounded, a host's within one unit in
        // the last place: per bin the relative difference of the shell volume
        // is at most (ulp(r+^3) + ulp(r-^3)) / (r+^3 - r-^3), plus the
        // roundings of the difference, the product and the divisions
        const double u = std::ldexp(1.0, -53);
        auto ulp = [](double x) {
            if (x == 0.0) return std::ldexp(1.0, -1074);
            int e;
            std::frexp(std::fabs(x), &e);
            return std::ldexp(1.0, e - 53);
        };
        double worst = 0.0;
        if (norm >= 1) {
            for (unsigned b = 0; b < p->nbin; ++b) {
                const double rm = (double)b * L.dr + L.r0, rp = (double)(b + 1) * L.dr + L.r0;
                const double cm = rm * rm * rm, cp = rp * rp * rp;
                const double d = std::fabs(cp - cm);
                const double e = d > 0.0 ? (ulp(cp) + ulp(cm)) * (1.0 + 4.0 * u) / d : INFINITY;
                worst = std::max(worst, e + (norm == 2 ? 8.0 : 6.0) * u);
            }
        }
        *rel_err_bound = worst;  // 0 for the buffer itself: bit for bit
    }
    return GOFR_OK;
}

// Device bytes one frame of natoms takes in a run: FP64 positions, FP32
// frames, the cell-sorted records and starts, with room for the boxes.
static size_t frame_device_bytes(size_t natoms)
{
    return padded_natoms(natoms) * (3 * 8 + 3 * 4 + 16 + 4 + 8) + 512;
}

int gofr_run_streamed(gofr_ctx *ctx, const double *positions, const double *boxes, int box_kind,
                      const int *type_ids, unsigned ntypes, size_t natoms, size_t nframes,
                      const gofr_params *p, size_t max_device_bytes,
                      unsigned long long *counts_host)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!p || !positions || !boxes || !type_ids || !counts_host)
        return fail(ctx, GOFR_ERR_ARG, "null argument");
    if (box_kind != GOFR_BOX_ORTHO && box_kind != GOFR_BOX_TRICLINIC)
        return fail(ctx, GOFR_ERR_ARG, "invalid box kind %d", box_kind);
    if (p->nparts > 1 && p->kernel != GOFR_KERNEL_AUTO && p->kernel != GOFR_KERNEL_F32_RECHECK &&
        p->kernel != GOFR_KERNEL_F64)
        return fail(ctx, GOFR_ERR_UNSUPPORTED, "per-partition counts need an all-pairs kernel");
    DevGuard g(ctx->device);
    // the whole calculation's shape, checked against every frame
    TrajDev whole;
    whole.T = nframes;
    whole.N = natoms;
    whole.ntypes = ntypes;
    RunShape rs;
    int rc = shape_of(ctx, whole, *p, rs);
    if (rc) return rc;
    const unsigned nparts = p->nparts > 1 ? p->nparts : 1;
    const size_t n_out = rs.data_length * nparts;
    const size_t stride = box_kind == GOFR_BOX_TRICLINIC ? 9 : 6;
    unsigned long long pairs = 0;
    double kernel_ms = 0.0;
    if (rs.n_lags > 0 && rs.n_orig > 0) {
        // origins per chunk: its frames [first origin, last origin + last lag]
        const size_t span = (size_t)(rs.n_lags - 1) * rs.every + 1;
        const size_t budget_frames = max_device_bytes / frame_device_bytes(natoms);
        if (budget_frames < span)
            return fail(ctx, GOFR_ERR_UNSUPPORTED,
                        "a device budget of %zu bytes holds %zu frames of %zu atoms, fewer than "
                        "the %zu frames of one origin's lags", max_device_bytes, budget_frames,
                        natoms, span);
        const size_t per_chunk = (budget_frames - span) / rs.skip + 1;
        std::vector<unsigned long long> chunk(n_out ? n_out : 1);
        std::vector<unsigned long long> total(n_out ? n_out : 1, 0ull);
        for (size_t k0 = 0; k0 < rs.n_orig; k0 += per_chunk) {
            const size_t k1 = std::min<size_t>(rs.n_orig, k0 + per_chunk);
            const size_t f0 = (size_t)p->primo + k0 * rs.skip;
            const size_t f1 = (size_t)p->primo + (k1 - 1) * rs.skip + span;
            ctx->trajs.resize(1);
            rc = upload_traj(ctx, ctx->trajs[0], positions + f0 * natoms * 3, boxes + f0 * stride,
                             box_kind, type_ids, ntypes, natoms, f1 - f0);
            if (rc) return rc;
            const TrajDev &t = ctx->trajs[0];
            // this chunk: origins 0, skip, ... of the uploaded frames, every lag
            gofr_params q = *p;
            q.primo = 0;
            RunShape rc_shape = rs;
            rc_shape.n_orig = (unsigned)(k1 - k0);
            Plan pl;
            rc = make_plan(ctx, t, q, pl, q.kernel != GOFR_KERNEL_TUNED);
            if (rc) return rc;
            if (pl.cells && q.kernel != GOFR_KERNEL_CELL && q.kernel != GOFR_KERNEL_CELL_WARP &&
                ensure_cells(ctx, t, pl) == GOFR_ERR_NOMEM) {
                ctx->err.clear();
                (void)cudaGetLastError();
                gofr_params a = q;
                a.kernel = GOFR_KERNEL_AUTO;
                Plan ap;
                rc = make_plan(ctx, t, a, ap, false);
                if (rc) return rc;
                pl = ap;
            }
            rc = ensure(ctx, ctx->d_counts, ctx->cap_counts, std::max<size_t>(n_out, 1));
            if (rc) return rc;
            CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
            CK(cudaMemsetAsync(ctx->d_stats, 0, ST_COUNT * sizeof(unsigned long long),
                               ctx->stream));
            if (n_out)
                CK(cudaMemsetAsync(ctx->d_counts, 0, n_out * sizeof(unsigned long long),
                                   ctx->stream));
            CK(cudaEventRecord(ctx->ev[1], ctx->stream));
            unsigned long long pw = 0;
            rc = enqueue_run(ctx, t, q, rc_shape, pl, ctx->d_counts, &pw);
            if (rc) return rc;
            CK(cudaEventRecord(ctx->ev[2], ctx->stream));
            if (n_out)
                CK(cudaMemcpyAsync(chunk.data(), ctx->d_counts, n_out * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            rc = check_device_error(ctx);
            if (rc) return rc;
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]) == cudaSuccess) kernel_ms += ms;
            for (size_t i = 0; i < n_out; ++i) total[i] += chunk[i];
            pairs += pw;
        }
        if (n_out) std::memcpy(counts_host, total.data(), n_out * sizeof(unsigned long long));
    } else if (n_out) {
        std::memset(counts_host, 0, n_out * sizeof(unsigned long long));
    }
    std::memset(&ctx->stats, 0, sizeof ctx->stats);
    ctx->stats.pairs = pairs;
    ctx->stats.evaluated = pairs;
    ctx->stats.kernel_ms = kernel_ms;
    ctx->stats.total_ms = kernel_ms;
    return GOFR_OK;
}

int gofr_sync(gofr_ctx *ctx)
{
    if (!ctx) return GOFR_ERR_ARG;
    DevGuard g(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = check_device_error(ctx);
    if (rc) return rc;
    unsigned long long st[ST_COUNT];
    CK(cudaMemcpy(st, ctx->d_stats, sizeof st, cudaMemcpyDeviceToHost));
    ctx->stats.candidates = st[ST_CANDIDATES];
    ctx->stats.rechecks = st[ST_RECHECKS];
    if (ctx->stats.kernel_used == GOFR_KERNEL_CELL ||
        ctx->stats.kernel_used == GOFR_KERNEL_CELL_WARP)
        ctx->stats.evaluated = st[ST_EVALUATED];
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]) == cudaSuccess) ctx->stats.kernel_ms = ms;
    if (cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[3]) == cudaSuccess) ctx->stats.total_ms = ms;
    return GOFR_OK;
}

int gofr_get_stats(const gofr_ctx *ctx, gofr_stats *out)
{
    if (!ctx || !out) return GOFR_ERR_ARG;
    *out = ctx->stats;
    out->launches = ctx->launches;
    out->h2d_bytes = ctx->h2d_bytes;
    return GOFR_OK;
}

int gofr_bin_thresholds(double rmin, double rmax, unsigned nbin, double *th)
{
    if (!th) return GOFR_ERR_ARG;
    if (!regular_bins(rmin, rmax, nbin)) return GOFR_ERR_UNSUPPORTED;
    BinMap bm(rmin, rmax, nbin);
    thresholds(bm, th);
    return GOFR_OK;
}

int gofr_plan_query(const double *box, int box_kind, const double *coord_min,
                    const double *coord_max, size_t natoms, unsigned ntypes,
                    const gofr_params *p, int *out)
{
    if (!box || !coord_min || !coord_max || !p || !out) return GOFR_ERR_ARG;
    if (box_kind != GOFR_BOX_ORTHO && box_kind != GOFR_BOX_TRICLINIC) return GOFR_ERR_ARG;
    if (natoms == 0 || ntypes == 0 || ntypes > 255) return GOFR_ERR_ARG;
    TrajDev t;
    t.T = 1;
    t.N = natoms;
    t.ntypes = ntypes;
    t.tric = box_kind == GOFR_BOX_TRICLINIC;
    std::vector<Box32> b32(1);
    if (!read_boxes(t, box, 1, t.tric ? 9 : 6, b32).empty()) return GOFR_ERR_ARG;
    for (int k = 0; k < 3; ++k) {
        if (!(coord_min[k] <= coord_max[k]) || !std::isfinite(coord_min[k]) ||
            !std::isfinite(coord_max[k]))
            return GOFR_ERR_ARG;
        set_extent(t, k, coord_min[k], coord_max[k]);
    }
    gofr_ctx ctx;  // host state only: the planner touches no device
    Plan pl;
    const int rc = make_plan(&ctx, t, *p, pl);
    for (int k = 0; k < 10; ++k) out[k] = 0;
    if (rc) return rc;
    out[0] = pl.kind == 1 ? GOFR_KERNEL_F64
                          : (pl.cellw ? GOFR_KERNEL_CELL_WARP
                                      : (pl.cells ? GOFR_KERNEL_CELL : GOFR_KERNEL_F32_RECHECK));
    if (pl.cells) {
        out[1] = pl.reach;
        for (int k = 0; k < 3; ++k) {
            out[2 + k] = pl.nc[k];
            out[5 + k] = pl.cellw ? pl.wblk[k] : pl.blk[k];
        }
        out[8] = pl.cellw ? pl.cta_warps : 0;
    }
    out[9] = pl.wrapcheck ? 1 : 0;
    return GOFR_OK;
}

int gofr_cellw_tables(const double *box, int box_kind, const double *coord_min,
                      const double *coord_max, double rmax, const int *nc, int *tables,
                      float *shifts, double *bound)
{
    if (!box || !coord_min || !coord_max || !nc || !tables) return GOFR_ERR_ARG;
    if (box_kind != GOFR_BOX_ORTHO && box_kind != GOFR_BOX_TRICLINIC) return GOFR_ERR_ARG;
    if (!(rmax > 0.0) || !std::isfinite(rmax)) return GOFR_ERR_ARG;
    TrajDev t;
    t.T = 1;
    t.N = 1;
    t.tric = box_kind == GOFR_BOX_TRICLINIC;
    std::vector<Box32> b32(1);
    if (!read_boxes(t, box, 1, t.tric ? 9 : 6, b32).empty()) return GOFR_ERR_ARG;
    for (int k = 0; k < 3; ++k) {
        if (!(coord_min[k] <= coord_max[k]) || !std::isfinite(coord_min[k]) ||
            !std::isfinite(coord_max[k]) || nc[k] < 1)
            return GOFR_ERR_ARG;
        set_extent(t, k, coord_min[k], coord_max[k]);
    }
    gofr_params p{};
    p.rmax = rmax;
    CellwGeom g;
    if (!cellw_geometry(t, p, nc, g)) return GOFR_ERR_UNSUPPORTED;
    tables[0] = g.nz_lo;
    tables[1] = g.nz_hi;
    for (int k = 0; k < 3; ++k) { tables[2 + k] = g.ny_lo[k]; tables[5 + k] = g.ny_hi[k]; }
    for (int k = 0; k < 15; ++k) { tables[8 + k] = g.nx_lo[k]; tables[23 + k] = g.nx_hi[k]; }
    if (shifts)
        for (int k = 0; k < CELLW_NSHIFT; ++k) {
            shifts[3 * k] = g.shift[k].x;
            shifts[3 * k + 1] = g.shift[k].y;
            shifts[3 * k + 2] = g.shift[k].z;
        }
    if (bound) {
        const Bound b = t.tric ? error_bound_cells_tric(t, g) : error_bound_cells(t);
        for (int k = 0; k < 3; ++k) bound[k] = b.e[k];
    }
    return GOFR_OK;
}

// incr added k times in sequence (lib/src/gofrt.cpp:118), in O(number of
// binades): within one binade of the running sum the rounded step is the
// same for every addition until the sum reaches the binade's upper end, so
// those additions are taken in one exact multiplication.  Exact ties (the
// step is half an ulp) are taken one at a time; they end in a fixed point.
static double repeated_sum(unsigned long long k, double incr)
{
    double s = 0.0;
    while (k > 0) {
        double n1 = s + incr;
        if (n1 == s) return s;  // the sum no longer moves
        if (s == 0.0 || !std::isfinite(n1)) { s = n1; --k; continue; }
        int e;
        std::frexp(s, &e);                     // s in [2^(e-1), 2^e)
        double top = std::ldexp(1.0, e);       // upper end of the binade
        double u = std::ldexp(1.0, e - 53);    // ulp in the binade
        double r = incr / u;                   // exact (power-of-two scaling)
        double fr = r - std::floor(r);
        if (fr == 0.5 || !(top - s > incr)) { s = n1; --k; continue; }
        double delta = n1 - s;                 // exact: same binade, Sterbenz
        // additions from s + j*delta stay exact steps while s + j*delta + incr <= top
        double jm = std::floor((top - s - incr) / delta) - 2.0;
        if (jm < 1.0) { s = n1; --k; continue; }
        unsigned long long j = jm >= (double)k ? k : (unsigned long long)jm;
        s = s + (double)j * delta;
        k -= j;
    }
    return s;
}

int gofr_counts_to_buffer(const unsigned long long *counts, size_t n, unsigned nparts,
                          unsigned ntimesteps, unsigned skip, double *out)
{
    if ((!counts || !out) && n) return GOFR_ERR_ARG;
    if (skip == 0) skip = 1;
    const double incr = (ntimesteps / skip > 0) ? 1.0 / (int)(ntimesteps / skip) : 1.0;
    if (nparts == 0) {
        for (size_t i = 0; i < n; ++i) out[i] = (double)counts[i] * incr;
        return GOFR_OK;
    }
    for (size_t i = 0; i < n; ++i) {
        double acc = repeated_sum(counts[i], incr);
        for (unsigned q = 1; q < nparts; ++q) acc += repeated_sum(counts[(size_t)q * n + i], incr);
        out[i] = acc;
    }
    return GOFR_OK;
}

// ---- batched trajectories ----------------------------------------------
int gofr_batch_set(gofr_ctx *ctx, const gofr_traj_desc *trajs, unsigned ntraj)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!trajs || ntraj == 0) return fail(ctx, GOFR_ERR_ARG, "empty batch");
    DevGuard g(ctx->device);
    for (auto &t : ctx->trajs) free_traj(t);
    free_batch(ctx);
    ctx->trajs.clear();
    ctx->trajs.resize(ntraj);
    size_t off = 0;
    for (unsigned k = 0; k < ntraj; ++k) {
        const gofr_traj_desc &d = trajs[k];
        int rc = upload_traj(ctx, ctx->trajs[k], d.positions, d.boxes, d.box_kind, d.type_ids,
                             d.ntypes, d.natoms, d.nframes);
        if (rc == GOFR_OK) {
            ctx->trajs[k].params = d.params;
            RunShape rs;
            rc = shape_of(ctx, ctx->trajs[k], d.params, rs);
            ctx->trajs[k].out_offset = off;
            ctx->trajs[k].out_count = rs.data_length;
            off += rs.data_length;
        }
        if (rc) {
            std::string m = ctx->err;
            for (auto &t : ctx->trajs) free_traj(t);
            ctx->trajs.clear();
            return fail(ctx, rc, "trajectory %u: %s", k, m.c_str());
        }
    }
    ctx->batch_total = off;
    int rc = GOFR_OK;
    if (dev_malloc(&ctx->batch.d_counts, std::max<size_t>(off, 1) * 8) != cudaSuccess)
        rc = fail(ctx, GOFR_ERR_NOMEM, "cannot allocate the batch counts");
    if (rc == GOFR_OK) rc = build_batch(ctx);
    if (rc) {
        std::string m = ctx->err;
        free_batch(ctx);
        for (auto &t : ctx->trajs) free_traj(t);
        ctx->trajs.clear();
        return fail(ctx, rc, "%s", m.c_str());
    }
    return GOFR_OK;
}

int gofr_batch_output_layout(const gofr_ctx *ctx, unsigned k, size_t *offset, size_t *n_counts)
{
    if (!ctx || !offset || !n_counts || k >= ctx->trajs.size()) return GOFR_ERR_ARG;
    *offset = ctx->trajs[k].out_offset;
    *n_counts = ctx->trajs[k].out_count;
    return GOFR_OK;
}

int gofr_batch_run(gofr_ctx *ctx, int use_graph, unsigned long long *counts_host)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!counts_host) return fail(ctx, GOFR_ERR_ARG, "null output buffer");
    if (ctx->trajs.empty() || !ctx->batch.h_stage)
        return fail(ctx, GOFR_ERR_STATE, "no batch uploaded");
    DevGuard g(ctx->device);
    auto &B = ctx->batch;
    if (use_graph && !B.graph) {
        cudaGraph_t graph = nullptr;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const unsigned long long launches_before = ctx->launches;
        int rc = enqueue_batch(ctx);
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
        ctx->launches = launches_before;
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess)
            return fail(ctx, GOFR_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&B.graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            B.graph = nullptr;
            return fail(ctx, GOFR_ERR_CUDA, "graph instantiation failed: %s",
                        cudaGetErrorString(e));
        }
    }
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    if (use_graph) {
        CK(cudaGraphLaunch(B.graph, ctx->stream));
        ctx->launches += (B.work[0].empty() ? 0 : 1) + (B.work[1].empty() ? 0 : 1) +
                         (B.cells.empty() ? 0 : 1) + B.f64_trajs.size() + B.cellw.size();
    } else {
        int rc = enqueue_batch(ctx);
        if (rc) return rc;
    }
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    std::memset(&ctx->stats, 0, sizeof ctx->stats);
    ctx->stats.pairs = B.pairs;
    ctx->stats.evaluated = B.pairs;
    const bool any_cells = !B.cells.empty() || !B.cellw.empty();
    ctx->stats.kernel_used = any_cells ? GOFR_KERNEL_CELL : GOFR_KERNEL_AUTO;
    int rc = gofr_sync(ctx);
    if (rc) return rc;
    // evaluated: every pair of the all-pairs members, the cell members' own count
    if (any_cells) ctx->stats.evaluated += B.allpairs_pairs;
    std::memcpy(counts_host, B.h_stage, ctx->batch_total * sizeof(unsigned long long));
    return GOFR_OK;
}

int gofr_set_centres(gofr_ctx *ctx, const double *centres, size_t nframes, unsigned ntypes)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!centres) return fail(ctx, GOFR_ERR_ARG, "null centres");
    if (ctx->trajs.size() != 1) return fail(ctx, GOFR_ERR_STATE, "no frames uploaded");
    TrajDev &t = ctx->trajs[0];
    if (nframes != t.T || ntypes != t.ntypes)
        return fail(ctx, GOFR_ERR_ARG, "centres are [%zu][%u][3], the frames need [%zu][%u][3]",
                    nframes, ntypes, t.T, t.ntypes);
    DevGuard g(ctx->device);
    cudaFree(t.d_cm);
    t.d_cm = nullptr;
    const size_t n = nframes * ntypes * 3;
    CK(dev_malloc(&t.d_cm, n * sizeof(double)));
    CK(cudaMemcpyAsync(t.d_cm, centres, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return GOFR_OK;
}

int gofr_msd_output_size(const gofr_ctx *ctx_c, const gofr_msd_params *p, size_t *n)
{
    gofr_ctx *ctx = const_cast<gofr_ctx *>(ctx_c);
    if (!ctx || !p || !n) return GOFR_ERR_ARG;
    if (ctx->trajs.size() != 1) return fail(ctx, GOFR_ERR_STATE, "no frames uploaded");
    const unsigned leff = (p->ntimesteps < p->tmax || p->tmax == 0) ? p->ntimesteps : p->tmax;
    *n = (size_t)leff * (p->center_of_mass ? 2 : 1) * ctx->trajs[0].ntypes;
    return GOFR_OK;
}

// MSD<T>::calc_init + calc_single_th (lib/src/msd.cpp:57-118) on the resident frames.
int gofr_msd_run(gofr_ctx *ctx, const gofr_msd_params *p, double *out_host)
{
    if (!ctx) return GOFR_ERR_ARG;
    if (!p) return fail(ctx, GOFR_ERR_ARG, "null params");
    if (ctx->trajs.size() != 1) return fail(ctx, GOFR_ERR_STATE, "no frames uploaded");
    const TrajDev &t = ctx->trajs[0];
    const unsigned skip = p->skip ? p->skip : 1;
    const unsigned leff = (p->ntimesteps < p->tmax || p->tmax == 0) ? p->ntimesteps : p->tmax;
    if ((unsigned long long)leff + p->ntimesteps + p->primo > (unsigned long long)t.T)
        return fail(ctx, GOFR_ERR_RANGE,
                    "trajectory is too short for this kind of calculation. Select a different "
                    "starting timestep or lower the size of the average or the lenght of the "
                    "time lag");
    if ((p->center_of_mass || p->in_center_of_mass_frame) && !t.d_cm)
        return fail(ctx, GOFR_ERR_STATE,
                    "the centre-of-mass options need the per-type centres (gofr_set_centres)");
    const int fk = (p->center_of_mass ? 2 : 1) * (int)t.ntypes;
    const size_t nout = (size_t)leff * fk;
    const unsigned n_orig = (p->ntimesteps + skip - 1) / skip;
    DevGuard g(ctx->device);
    std::memset(&ctx->stats, 0, sizeof ctx->stats);
    if (nout == 0) return GOFR_OK;
    if (n_orig == 0) {  // no origin: the reference leaves its zeroed buffer
        std::memset(out_host, 0, nout * sizeof(double));
        return GOFR_OK;
    }
    int rc = ensure(ctx, ctx->d_msd_partial, ctx->cap_msd_partial, nout * n_orig);
    if (rc) return rc;
    rc = ensure(ctx, ctx->d_msd_out, ctx->cap_msd_out, nout);
    if (rc) return rc;
    MsdLaunch M{};
    M.pos64 = t.pos64;
    M.cm = t.d_cm;
    M.perm = t.d_perm;
    M.tbegin = t.d_tbegin;
    M.partial = ctx->d_msd_partial;
    M.N = (int)t.N;
    M.ntypes = (int)t.ntypes;
    M.leff = (int)leff;
    M.n_orig = (int)n_orig;
    M.skip = (int)skip;
    M.primo = (long long)p->primo;
    M.cm_msd = p->center_of_mass ? 1 : 0;
    M.cm_self = p->in_center_of_mass_frame ? 1 : 0;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_stats, 0, ST_COUNT * sizeof(unsigned long long), ctx->stream));
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    ctx->launches += 2;
    if (launch_msd(M, ctx->d_msd_out, ctx->num_sms, ctx->stream))
        return fail(ctx, GOFR_ERR_CUDA, "MSD kernel launch failed: %s",
                    cudaGetErrorString(cudaGetLastError()));
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    CK(cudaMemcpyAsync(out_host, ctx->d_msd_out, nout * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    // one squared displacement per (lag, origin, atom)
    ctx->stats.pairs = (unsigned long long)leff * n_orig * t.N;
    ctx->stats.evaluated = ctx->stats.pairs;
    ctx->stats.kernel_used = -1;
    return gofr_sync(ctx);
}

int gofr_neigh_layout(const gofr_ctx *ctx_c, const gofr_neigh_spec *spec, unsigned nspec,
                      size_t *list_len, size_t *rpos_len)
{
    gofr_ctx *ctx = const_cast<gofr_ctx *>(ctx_c);
    if (!ctx || !list_len || !rpos_len || (nspec && !spec)) return GOFR_ERR_ARG;
    if (ctx->trajs.size() != 1) return fail(ctx, GOFR_ERR_STATE, "no frames uploaded");
    const TrajDev &t = ctx->trajs[0];
    if (nspec != t.ntypes)
        return fail(ctx, GOFR_ERR_ARG,
                    "In neighbours list you must specify parameters for each atomic type");
    unsigned long long tot = 0;
    for (unsigned k = 0; k < nspec; ++k) tot += spec[k].nneigh;
    *list_len = t.N * (size_t)(tot + nspec);
    *rpos_len = t.N * (size_t)4 * tot;
    return GOFR_OK;
}

// Neighbours::update_neigh(timestep, sort) (lib/src/neighbour.cpp:9-79).
int gofr_neigh_run(gofr_ctx *ctx, const gofr_neigh_spec *spec, unsigned nspec, size_t timestep,
                   int sort, unsigned long long *list_host, double *rpos_host)
{
    size_t list_len = 0, rpos_len = 0;
    int rc = gofr_neigh_layout(ctx, spec, nspec, &list_len, &rpos_len);
    if (rc) return rc;
    const TrajDev &t = ctx->trajs[0];
    if (timestep >= t.T)
        return fail(ctx, GOFR_ERR_ARG, "timestep %zu outside the %zu frames", timestep, t.T);
    if (nspec > (unsigned)NEIGH_MAXT)
        return fail(ctx, GOFR_ERR_UNSUPPORTED, "neighbour lists support at most %d types",
                    NEIGH_MAXT);
    if (t.N > (size_t)INT32_MAX / 2) return fail(ctx, GOFR_ERR_UNSUPPORTED, "too many atoms");
    if ((list_len && !list_host) || (rpos_len && !rpos_host))
        return fail(ctx, GOFR_ERR_ARG, "null output");
    DevGuard g(ctx->device);
    // meta: nneigh[nt], loff[nt], roff[nt], flags (u32 in a u64), first_err
    const unsigned nt = nspec;
    std::vector<unsigned long long> meta(3 * nt + 2, 0ull);
    std::vector<double> cut2(nt);
    unsigned long long lo = 0, ro = 0;
    for (unsigned k = 0; k < nt; ++k) {
        meta[k] = spec[k].nneigh;
        meta[nt + k] = lo;
        meta[2 * nt + k] = ro;
        lo += (spec[k].nneigh + 1) * (unsigned long long)t.N;
        ro += spec[k].nneigh * (unsigned long long)t.N * 4;
        cut2[k] = spec[k].cut2;
    }
    meta[3 * nt + 1] = ~0ull;
    rc = ensure(ctx, ctx->d_nl_meta, ctx->cap_nl_meta, meta.size());
    if (!rc) rc = ensure(ctx, ctx->d_nl_cut2, ctx->cap_nl_cut2, std::max<size_t>(nt, 1));
    if (!rc) rc = ensure(ctx, ctx->d_nl_list, ctx->cap_nl_list, std::max<size_t>(list_len, 1));
    if (!rc) rc = ensure(ctx, ctx->d_nl_rpos, ctx->cap_nl_rpos, std::max<size_t>(rpos_len, 1));
    if (!rc) rc = ensure(ctx, ctx->d_nl_full, ctx->cap_nl_full, std::max<size_t>(t.N * nt, 1));
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_nl_meta, meta.data(), meta.size() * 8, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_nl_cut2, cut2.data(), nt * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
    if (list_len) CK(cudaMemsetAsync(ctx->d_nl_list, 0, list_len * 8, ctx->stream));
    if (rpos_len) CK(cudaMemsetAsync(ctx->d_nl_rpos, 0, rpos_len * 8, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_stats, 0, ST_COUNT * sizeof(unsigned long long), ctx->stream));
    NeighLaunch L{};
    L.pos64 = t.pos64;
    L.box64 = t.box64;
    L.types = t.types;
    L.nneigh = ctx->d_nl_meta;
    L.loff = ctx->d_nl_meta + nt;
    L.roff = ctx->d_nl_meta + 2 * nt;
    L.cut2 = ctx->d_nl_cut2;
    L.list = ctx->d_nl_list;
    L.rpos = ctx->d_nl_rpos;
    L.full = ctx->d_nl_full;
    L.flags = reinterpret_cast<unsigned *>(ctx->d_nl_meta + 3 * nt);
    L.first_err = ctx->d_nl_meta + 3 * nt + 1;
    L.err = ctx->d_err;
    L.N = (int)t.N;
    L.ntypes = (int)nt;
    L.timestep = (long long)timestep;
    L.tric = t.tric;
    // FP32 prefilter with the all-pairs kernel's certified bound, where the
    // minimum image of the near pairs is certain
    double cmax = -INFINITY;
    for (unsigned k = 0; k < nt; ++k) cmax = std::max(cmax, cut2[k]);
    {
        if (std::isfinite(cmax) && cmax >= 0.0) {
            const Bound b = error_bound(t);
            const float hi = f_up(cmax + Efun(b, cmax));
            const double emax = std::max(b.e[0], std::max(b.e[1], b.e[2]));
            const double reach = std::sqrt((double)hi) * (1.0 + std::ldexp(1.0, -20)) +
                                 2.0 * emax + 1e-9;
            if (std::isfinite(hi) && t.bs.lh_min > reach) {
                L.prefilter = 1;
                L.hi_f = hi;
                L.pos32 = t.pos32;
                L.box32 = t.box32;
                L.NP = (long long)padded_natoms(t.N);
            }
        }
    }
    // Cell-list form: orthorhombic boxes constant over the trajectory, cells
    // of edge >= the largest cutoff (x (1 + 1e-6)), at least 3 per axis.
    // ANALISI_GB300_NEIGH_KERNEL=allpairs keeps the all-pairs form.
    {
        const char *env = std::getenv("ANALISI_GB300_NEIGH_KERNEL");
        const bool allpairs = env && std::strcmp(env, "allpairs") == 0;
        gofr_params q{};
        q.rmax = cmax > 0.0 ? std::sqrt(cmax) : 0.0;
        int nc[3];
        if (!allpairs && L.prefilter && !t.tric && t.box_constant && t.N < (1u << 24) &&
            q.rmax > 0.0 && cell_grid(t, q, 1, nc)) {
            Plan pl;
            for (int k = 0; k < 3; ++k) pl.nc[k] = nc[k];
            const int crc = ensure_cells(ctx, t, pl);
            if (crc == GOFR_OK) {
                const size_t ncell = (size_t)nc[0] * nc[1] * nc[2];
                L.cells = 1;
                for (int k = 0; k < 3; ++k) L.nc[k] = nc[k];
                L.cstart = t.d_cstart + timestep * (ncell + 1);
                L.csidt = t.d_sidt + timestep * padded_natoms(t.N);
            } else if (crc == GOFR_ERR_NOMEM) {
                // no room for the cell lists: the all-pairs form (and the failed
                // allocation's error is not a later launch's)
                ctx->err.clear();
                (void)cudaGetLastError();
            } else {
                return crc;  // a failed cell build is a device error, not a shortage
            }
        }
    }
    std::memset(&ctx->stats, 0, sizeof ctx->stats);
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    ++ctx->launches;
    if (launch_neigh_build(L, ctx->num_sms, ctx->stream))
        return fail(ctx, GOFR_ERR_CUDA, "neighbour-list kernel launch failed: %s",
                    cudaGetErrorString(cudaGetLastError()));
    unsigned long long tail[2] = {0ull, 0ull};
    CK(cudaMemcpyAsync(tail, ctx->d_nl_meta + 3 * nt, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (tail[0] & 2ull) {
        // a cell neighbourhood held more survivors than a warp's buffer: the
        // all-pairs form over again
        L.cells = 0;
        CK(cudaMemcpyAsync(ctx->d_nl_meta + 3 * nt, meta.data() + 3 * nt, 16,
                           cudaMemcpyHostToDevice, ctx->stream));
        if (list_len) CK(cudaMemsetAsync(ctx->d_nl_list, 0, list_len * 8, ctx->stream));
        if (rpos_len) CK(cudaMemsetAsync(ctx->d_nl_rpos, 0, rpos_len * 8, ctx->stream));
        ++ctx->launches;
        if (launch_neigh_build(L, ctx->num_sms, ctx->stream))
            return fail(ctx, GOFR_ERR_CUDA, "neighbour-list kernel launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
        CK(cudaMemcpyAsync(tail, ctx->d_nl_meta + 3 * nt, 16, cudaMemcpyDeviceToHost,
                           ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    if (tail[0] & 1ull) {  // some list is full: look for the reference's overflow
        ++ctx->launches;
        if (launch_neigh_check(L, ctx->num_sms, ctx->stream))
            return fail(ctx, GOFR_ERR_CUDA, "neighbour-list check launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
        CK(cudaMemcpyAsync(tail, ctx->d_nl_meta + 3 * nt, 16, cudaMemcpyDeviceToHost,
                           ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    const bool overflow = tail[1] != ~0ull;
    if (!overflow && sort) {
        ++ctx->launches;
        if (launch_neigh_sort(L, ctx->num_sms, ctx->stream))
            return fail(ctx, GOFR_ERR_CUDA, "neighbour-list sort launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
    }
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    if (list_len)
        CK(cudaMemcpyAsync(list_host, ctx->d_nl_list, list_len * 8, cudaMemcpyDeviceToHost,
                           ctx->stream));
    if (rpos_len)
        CK(cudaMemcpyAsync(rpos_host, ctx->d_nl_rpos, rpos_len * 8, cudaMemcpyDeviceToHost,
                           ctx->stream));
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    ctx->stats.pairs = (unsigned long long)t.N * t.N;
    ctx->stats.evaluated = ctx->stats.pairs;
    ctx->stats.kernel_used = L.cells ? -2 : -1;  // neighbour lists: -2 cell-list form
    rc = gofr_sync(ctx);
    if (rc) return rc;
    if (overflow) {
        // the reference's message: sizes of the two lists when the pair came
        const unsigned long long i = tail[1] / t.N, j = tail[1] % t.N;
        const unsigned ti = (unsigned)t.h_types[i], tj = (unsigned)t.h_types[j];
        auto before = [&](unsigned long long a, unsigned k, unsigned long long lim) {
            const unsigned long long *l = list_host + meta[nt + k] + a * (spec[k].nneigh + 1);
            unsigned long long n = 0;
            for (unsigned long long q = 0; q < l[0]; ++q) n += l[1 + q] < lim ? 1 : 0;
            return n;
        };
        return fail(ctx, GOFR_ERR_NEIGH_FULL,
                    "Too many neighbours in shell! (iatom=%llu jatom=%llu ni=%llu nj=%llu "
                    "itype=%u jtype=%u)",
                    i, j, before(i, tj, j), before(j, ti, i), ti, tj);
    }
    return GOFR_OK;
}

}  // extern "C"
