// Cell-list form of the FP32 + FP64-recheck pair kernel, for large N.
//
// The reference evaluates all N^2 ordered pairs per (lag, origin)
// (lib/src/gofrt.cpp:101-102).  Here, for orthorhombic boxes that do not
// change over the trajectory, every frame's atoms are binned into a grid of
// cells whose edge is at least rmax (plus a margin): a pair at minimum-image
// distance <= rmax always lies in cells that are neighbours (periodically) in
// every axis, so pairs outside the neighbourhood are never counted by the
// reference and need not be evaluated.  Every pair inside the neighbourhood
// goes through exactly the same certified FP32 test and FP64 recheck as the
// all-pairs kernel, so the counts are identical.
//
// Cells have edge >= rmax / reach (reach 1 or 2), so such a pair lies at most
// `reach` cells apart on every axis.  Layout per frame: atoms sorted by cell
// (x fastest); FP32 SoA x|y|z of the coordinates wrapped into the box in FP64
// (x - n L, n = floor((x - xlo) / L)) and rounded about the box centre; a
// u32 word type << 24 | original atom id; and the cell start offsets.  A work
// item is (lag, origin, block of bx*by*bz cells): the block's atoms at the
// origin frame against the atoms of the block's neighbourhood
// ((bx+2 reach)(by+2 reach)(bz+2 reach) cells, never more than the box holds,
// so every cell appears once) at the lagged frame.  A neighbour cell reached
// across the box boundary is the periodic image of that cell: its atoms are
// shifted by +-fl32(L) on that axis when they enter shared memory, so the
// pair arithmetic is a plain FP32 difference and d2 (6 operations per two
// pairs as f32x2), the minimum image being the image the neighbourhood
// selects.  The host certifies these FP32 values with their own error bound
// (gofr_capi.cu, error_bound_cells), then every candidate goes through the
// same window test and FP64 recheck as in the all-pairs kernel.
#include <cstdint>
#include <cuda_runtime.h>

#include "gofr_device.cuh"
#include "gofr_internal.h"

namespace gofr {

namespace cells {

constexpr int NT = 256;
constexpr int TJ = 1024;      // second atoms per shared-memory tile
constexpr int SLOTS = 16;
constexpr int QCAP = 1024;
constexpr int MAXR = 128;     // max contiguous ranges of a neighbourhood (checked on host)
constexpr int FLUSH_ILP = 2;  // slots binned per round of a warp flush
static_assert(SLOTS % FLUSH_ILP == 0, "a flush round reads rows q0 .. q0 + FLUSH_ILP - 1 < SLOTS");

typedef unsigned long long f2;
__device__ __forceinline__ f2 f2pk(float a, float b)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2up(f2 v, float &a, float &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2 f2sub(f2 a, f2 b)
{
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2mul(f2 a, f2 b)
{
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2fma(f2 a, f2 b, f2 c)
{
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// d2 of (i, j0) and (i, j1) for second atoms already in the first atom's
// image: three differences, then one multiply and two FMAs, as f32x2.
__device__ __forceinline__ f2 pair2s(f2 xi, f2 yi, f2 zi, f2 xj, f2 yj, f2 zj)
{
    const f2 dx = f2sub(xi, xj), dy = f2sub(yi, yj), dz = f2sub(zi, zj);
    f2 d2 = f2mul(dx, dx);
    d2 = f2fma(dy, dy, d2);
    d2 = f2fma(dz, dz, d2);
    return d2;
}

__device__ __forceinline__ int wrapi(int a, int n)
{
    a %= n;
    return a < 0 ? a + n : a;
}

// ---------------------------------------------------------------------------
// cell build
// ---------------------------------------------------------------------------
// tric: the cell of the coordinates reduced into the axis-aligned cell by
// the lattice (wrap_tric64, as the warp-streamed records are), else of the
// fractional part of each coordinate's quotient.
__global__ void k_cell_assign(const double *__restrict__ pos, size_t T, size_t N, double xlo,
                              double ylo, double zlo, double Lx, double Ly, double Lz, double xy,
                              double xz, double yz, int tric, int ncx, int ncy, int ncz,
                              int *__restrict__ cell_of, int *__restrict__ rank_of,
                              int *__restrict__ count)
{
    const int ncell = ncx * ncy * ncz;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < T * N;
         g += (size_t)gridDim.x * blockDim.x) {
        const size_t f = g / N;
        const double *p = pos + g * 3;
        const int nc[3] = {ncx, ncy, ncz};
        int c[3];
        if (tric) {
            const double lo[3] = {xlo, ylo, zlo}, L[3] = {Lx, Ly, Lz}, tilt[3] = {xy, xz, yz};
            double w[3];
            wrap_tric64(p, lo, L, tilt, w);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double u = __ddiv_rn(__dsub_rn(w[k], lo[k]), L[k]);
                const int ck = (int)floor(u * nc[k]);
                c[k] = ck < 0 ? 0 : (ck >= nc[k] ? nc[k] - 1 : ck);
            }
        } else {
            double u[3] = {__ddiv_rn(__dsub_rn(p[0], xlo), Lx), __ddiv_rn(__dsub_rn(p[1], ylo), Ly),
                           __ddiv_rn(__dsub_rn(p[2], zlo), Lz)};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double w = u[k] - floor(u[k]);
                int ck = (int)(w * nc[k]);
                c[k] = ck < 0 ? 0 : (ck >= nc[k] ? nc[k] - 1 : ck);
            }
        }
        const int cell = (c[2] * ncy + c[1]) * ncx + c[0];
        cell_of[g] = cell;
        rank_of[g] = atomicAdd(count + f * (size_t)(ncell + 1) + cell, 1);
    }
}

// exclusive scan of each frame's counts into starts (one CTA per frame)
__global__ void k_cell_scan(const int *__restrict__ count, int *__restrict__ start, int ncell)
{
    __shared__ int part[NT];
    const size_t f = blockIdx.x;
    const int *c = count + f * (size_t)(ncell + 1);
    int *s = start + f * (size_t)(ncell + 1);
    const int per = (ncell + NT - 1) / NT;
    const int b0 = threadIdx.x * per, b1 = min(ncell, b0 + per);
    int sum = 0;
    for (int i = b0; i < b1; ++i) sum += c[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < NT; ++t) {
            const int v = part[t];
            part[t] = run;
            run += v;
        }
        s[ncell] = run;
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int i = b0; i < b1; ++i) {
        s[i] = run;
        run += c[i];
    }
}

// Sorted copy of every frame.  Coordinates: w = x - n L with n = floor((x -
// xlo) / L) (the n of the cell assignment), one FMA in FP64, then
// fl32(fl64(w - c)) with c the box centre.
__global__ void k_cell_scatter(const double *__restrict__ pos64,
                               const unsigned char *__restrict__ types8, size_t T, size_t N,
                               size_t NP, int ncell, double xlo, double ylo, double zlo, double Lx,
                               double Ly, double Lz, double cx, double cy, double cz,
                               const int *__restrict__ cell_of, const int *__restrict__ rank_of,
                               const int *__restrict__ start, float *__restrict__ spos,
                               unsigned *__restrict__ sidt)
{
    const double lo[3] = {xlo, ylo, zlo}, L[3] = {Lx, Ly, Lz}, c[3] = {cx, cy, cz};
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < T * N;
         g += (size_t)gridDim.x * blockDim.x) {
        const size_t f = g / N, a = g - f * N;
        const size_t d = (size_t)start[f * (size_t)(ncell + 1) + cell_of[g]] + rank_of[g];
        const double *p = pos64 + g * 3;
        float *dst = spos + f * 3 * NP;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double n = floor(__ddiv_rn(__dsub_rn(p[k], lo[k]), L[k]));
            const double w = __fma_rn(-n, L[k], p[k]);
            dst[k * NP + d] = __double2float_rn(__dsub_rn(w, c[k]));
        }
        sidt[f * NP + d] = ((unsigned)types8[a] << 24) | (unsigned)a;
    }
}

// ---------------------------------------------------------------------------
// pair kernel
// ---------------------------------------------------------------------------
struct Range {
    int begin, end;   // sorted atom indices [begin, end)
    int shift;        // image of the cells: (sx+1) | (sy+1) << 2 | (sz+1) << 4, s in {-1,0,1}
};

__device__ __forceinline__ int image_of(int c, int n) { return c < 0 ? -1 : (c >= n ? 1 : 0); }

// Rows of contiguous atom ranges making up a set of cells, with the periodic
// image each row segment is reached in.  Cells [x0, x0+nx) x [y0, y0+ny) x
// [z0, z0+nz) in unwrapped coordinates, nx <= ncx, ny <= ncy, nz <= ncz (each
// cell at most once).
__device__ int build_ranges(const int *start, int ncx, int ncy, int ncz, int x0, int nx, int y0,
                            int ny, int z0, int nz, Range *out)
{
    int n = 0;
    for (int dz = 0; dz < nz; ++dz) {
        const int uz = z0 + dz, cz = wrapi(uz, ncz);
        for (int dy = 0; dy < ny; ++dy) {
            const int uy = y0 + dy, cy = wrapi(uy, ncy);
            const int rowbase = (cz * ncy + cy) * ncx;
            const int yz = (image_of(uy, ncy) + 1) << 2 | (image_of(uz, ncz) + 1) << 4;
            const int a = wrapi(x0, ncx);
            const int b = a + nx;  // exclusive, may pass the row end
            // the first segment starts at x0 (image of x0), a wrapped second
            // segment is one image further
            const int sx0 = image_of(x0, ncx);
            if (b <= ncx) {
                out[n++] = {start[rowbase + a], start[rowbase + b], (sx0 + 1) | yz};
            } else {
                out[n++] = {start[rowbase + a], start[rowbase + ncx], (sx0 + 1) | yz};
                out[n++] = {start[rowbase], start[rowbase + (b - ncx)], (sx0 + 2) | yz};
            }
        }
    }
    return n;
}

// flat index q of a range list -> range (binary search of the prefix table:
// the last range r with pre[r] <= q); the atom is rg[r].begin + q - pre[r]
__device__ __forceinline__ int range_of(const int *pre, int nr, int q)
{
    int lo = 0, hi = nr - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// 4-byte asynchronous global -> shared copy (no register staging).
__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Work items are (lag, origin, block of cells), block fastest, handed to the
// CTAs round-robin: the CTAs running at one time share a few frames, which
// stay in L2.  Each item streams its neighbourhood atoms through two
// shared-memory tiles, the next one copied asynchronously while the current
// one is evaluated.
//
// MULTI: the items of several trajectories in one launch (Cs, item_end in
// device memory, the current trajectory's record copied to shared memory);
// otherwise one trajectory whose record Cp stays in the kernel parameters,
// which instructions read directly (no registers held for them).
template <int R, bool MULTI>
__global__ void __launch_bounds__(NT, 2)
    k_pairs_cell(const CellLaunch Cp, const CellLaunch *__restrict__ Cs,
                 const long long *__restrict__ item_end, int nmem, int win_cap, int hist_cap)
{
    constexpr int TI = NT * R;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ CellLaunch sC;  // the trajectory of the current items (MULTI)
    const CellLaunch &C = MULTI ? sC : Cp;
    const PairLaunch &P = C.pair;
    unsigned *jbuf = reinterpret_cast<unsigned *>(smem);          // [2][x|y|z|id-type][TJ]
    uint2 *slots = reinterpret_cast<uint2 *>(jbuf + 2 * 4 * TJ);  // [SLOTS][NT]
    uint4 *rq = reinterpret_cast<uint4 *>(slots + SLOTS * NT);    // [QCAP]
    float2 *win = reinterpret_cast<float2 *>(rq + QCAP);          // [win_cap]
    unsigned *hist = reinterpret_cast<unsigned *>(win + win_cap); // [hist_cap]
    unsigned short *chtab = reinterpret_cast<unsigned short *>(hist + hist_cap);
    __shared__ Range irg[MAXR], jrg[MAXR];
    __shared__ int ipre[MAXR + 1], jpre[MAXR + 1];
    __shared__ int nir, njr, rqn;
    // type << 24 | atom id of this pass's first atoms, read by the flush
    // (a shared load in place of an R-way register select)
    __shared__ unsigned s_iv[R][NT];

    // the current trajectory's item range (kept in shared memory: the pair
    // loop needs every register)
    __shared__ long long s_begin, s_end;
    __shared__ int s_m;

    const int tid = threadIdx.x;
    float L32[3];
    int cur_lag = -1;
    long long pairs_since = 0;
    unsigned long long n_cand = 0, n_rech = 0, n_eval = 0;
    uint2 *const my_slots = slots + tid;
    const long long total = MULTI ? (nmem > 0 ? item_end[nmem - 1] : 0) : Cp.pair.n_items;
    if (tid == 0) {
        s_m = -1;
        s_begin = 0;
        s_end = MULTI ? 0 : total;
    }
    if (!MULTI) {
        for (int i = tid; i < P.nbin; i += NT) win[i] = P.win[i];
        for (int i = tid; i < P.nch * P.nbin; i += NT) hist[i] = 0u;
        for (int i = tid; i < P.ntypes * P.ntypes; i += NT) chtab[i] = P.chtab[i];
        if (tid == 0) rqn = 0;
    }
    __syncthreads();

    // adds the shared histogram of the current (trajectory, lag) to its counts
    auto flush_hist = [&]() {
        const int hlen = P.nch * P.nbin;
        for (int i = tid; i < hlen; i += NT) {
            const unsigned v = hist[i];
            if (v) {
                atomicAdd(P.counts + (long long)cur_lag * P.every * hlen + i, (unsigned long long)v);
                hist[i] = 0u;
            }
        }
    };

    for (long long g = blockIdx.x; g < total; g += gridDim.x) {
        if (MULTI && g >= s_end) {  // next trajectory (the same decision in every thread)
            __syncthreads();
            if (cur_lag >= 0) flush_hist();
            __syncthreads();
            if (tid == 0) {
                int m = s_m;
                long long b = s_begin, e = s_end;
                while (g >= e) {
                    ++m;
                    b = e;
                    e = item_end[m];
                }
                s_m = m;
                s_begin = b;
                s_end = e;
            }
            __syncthreads();
            {
                const int *src = reinterpret_cast<const int *>(Cs + s_m);
                int *dst = reinterpret_cast<int *>(&sC);
                for (int i = tid; i < (int)(sizeof(CellLaunch) / sizeof(int)); i += NT) dst[i] = src[i];
            }
            __syncthreads();
            for (int i = tid; i < P.nbin; i += NT) win[i] = P.win[i];
            for (int i = tid; i < P.nch * P.nbin; i += NT) hist[i] = 0u;
            for (int i = tid; i < P.ntypes * P.ntypes; i += NT) chtab[i] = P.chtab[i];
            if (tid == 0) rqn = 0;
            cur_lag = -1;
            pairs_since = 0;
            __syncthreads();
        }
        const long long item = MULTI ? g - s_begin : g;
        const int nbx = C.nb[0], nby = C.nb[1], nbz = C.nb[2];
        const long long nblocks = (long long)nbx * nby * nbz;
        const long long per_lag = nblocks * P.n_orig;
        const long long NP = P.NP;
        const int ncell = C.nc[0] * C.nc[1] * C.nc[2];
        const float hi_f = P.hi_f;
        const int half = P.nch / 2;
        const int lag_idx = (int)(item / per_lag);
        const long long rem = item - (long long)lag_idx * per_lag;
        const int k = (int)(rem / nblocks);
        const int blk = (int)(rem - (long long)k * nblocks);
        const long long fo = P.primo + (long long)k * P.skip;
        const long long fl = fo + (long long)lag_idx * P.every;
        {
            const Box32 b = P.box32[fo];  // the box is the same in every frame
#pragma unroll
            for (int a = 0; a < 3; ++a) L32[a] = b.L[a];
        }
        const int bz = blk / (nbx * nby), by = (blk / nbx) % nby, bx = blk % nbx;
        const int cx0 = bx * C.b[0], cy0 = by * C.b[1], cz0 = bz * C.b[2];
        const int cnx = min(C.b[0], C.nc[0] - cx0), cny = min(C.b[1], C.nc[1] - cy0),
                  cnz = min(C.b[2], C.nc[2] - cz0);
        __syncthreads();  // previous item done with the range tables and tiles
        if (tid == 0) {
            const int *st_o = C.start + fo * (size_t)(ncell + 1);
            const int *st_l = C.start + fl * (size_t)(ncell + 1);
            nir = build_ranges(st_o, C.nc[0], C.nc[1], C.nc[2], cx0, cnx, cy0, cny, cz0, cnz, irg);
            // b + 2 reach <= nc on every axis (host plan): each cell once
            const int m = C.reach;
            njr = build_ranges(st_l, C.nc[0], C.nc[1], C.nc[2], cx0 - m, cnx + 2 * m, cy0 - m,
                               cny + 2 * m, cz0 - m, cnz + 2 * m, jrg);
            if (!GOFR_CHECK(nir <= MAXR && njr <= MAXR, P.err)) nir = njr = 0;
            ipre[0] = 0;
            for (int r = 0; r < nir; ++r) ipre[r + 1] = ipre[r] + (irg[r].end - irg[r].begin);
            jpre[0] = 0;
            for (int r = 0; r < njr; ++r) jpre[r + 1] = jpre[r] + (jrg[r].end - jrg[r].begin);
        }
        __syncthreads();
        {
            // flush when the lag changes, or before a u32 shared bin could
            // overflow: one item adds at most n_i*n_j hits to a bin
            const long long pairs_item = (long long)ipre[nir] * jpre[njr];
            if (lag_idx != cur_lag || pairs_since + pairs_item >= (1ll << 31)) {
                if (cur_lag >= 0) {
                    flush_hist();
                    __syncthreads();
                }
                cur_lag = lag_idx;
                pairs_since = 0;
            }
            pairs_since += pairs_item;
        }
        const int n_i = ipre[nir], n_j = jpre[njr];
        n_eval += (tid == 0) ? (unsigned long long)n_i * n_j : 0ull;
        const float *fo32 = C.spos + fo * 3 * NP;
        const float *fl32 = C.spos + fl * 3 * NP;
        const unsigned *fo_idt = C.sidt + fo * NP;
        const unsigned *fl_idt = C.sidt + fl * NP;
        const int ntile = (n_j + TJ - 1) / TJ;

        // Copies tile t of the neighbourhood into buffer t & 1 (all threads;
        // thread tid takes elements tid + k NT, k < TJ / NT) and returns the
        // image codes of this thread's elements, 6 bits each.
        auto load_tile = [&](int t) -> unsigned {
            const int jbase = t * TJ;
            const int tj = min(TJ, n_j - jbase);
            unsigned *dst = jbuf + (t & 1) * 4 * TJ;
            unsigned codes = 0u;
#pragma unroll
            for (int e = 0; e < TJ / NT; ++e) {
                const int q = tid + e * NT;
                if (q < tj) {
                    const int r = range_of(jpre, njr, jbase + q);
                    const int s = jrg[r].begin + (jbase + q - jpre[r]);
                    codes |= (unsigned)jrg[r].shift << (6 * e);
                    cp_async4(dst + q, fl32 + s);
                    cp_async4(dst + TJ + q, fl32 + NP + s);
                    cp_async4(dst + 2 * TJ + q, fl32 + 2 * NP + s);
                    cp_async4(dst + 3 * TJ + q, fl_idt + s);
                } else if (q < ((tj + 3) & ~3)) {
                    // no atom: NaN never passes d2 <= hi_f
                    dst[q] = dst[TJ + q] = dst[2 * TJ + q] = 0x7fc00000u;
                    dst[3 * TJ + q] = 0xffffffffu;
                }
            }
            cp_async_commit();
            return codes;
        };
        // Moves this thread's elements of tile t (copies complete) to the
        // image of their cell: x += s fl32(L), one FP32 rounding.
        auto shift_tile = [&](int t, unsigned codes) {
            const int tj = min(TJ, n_j - t * TJ);
            float *xs = reinterpret_cast<float *>(jbuf + (t & 1) * 4 * TJ);
#pragma unroll
            for (int e = 0; e < TJ / NT; ++e) {
                const int q = tid + e * NT;
                const unsigned c = (codes >> (6 * e)) & 63u;
                if (q < tj && c != 21u) {  // 21: image (0, 0, 0)
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const int sa = (int)((c >> (2 * a)) & 3u) - 1;
                        if (sa) xs[a * TJ + q] = __fadd_rn(xs[a * TJ + q], sa > 0 ? L32[a] : -L32[a]);
                    }
                }
            }
        };

        for (int ibase = 0; ibase < n_i; ibase += TI) {
            f2 xi[R], yi[R], zi[R];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int q = ibase + r * NT + tid;
                float x, y, z;
                if (q < n_i) {
                    const int rr = range_of(ipre, nir, q);
                    const int s = irg[rr].begin + (q - ipre[rr]);  // block cells: image (0,0,0)
                    x = fo32[s]; y = fo32[NP + s]; z = fo32[2 * NP + s];
                    s_iv[r][tid] = fo_idt[s];
                } else {
                    x = y = z = __int_as_float(0x7fc00000);
                    s_iv[r][tid] = 0x00ffffffu;  // type 0, no atom id
                }
                xi[r] = f2pk(x, x); yi[r] = f2pk(y, y); zi[r] = f2pk(z, z);
            }
            int cnt = 0;
            unsigned codes = load_tile(0);
            for (int t = 0; t < ntile; ++t) {
                const int tj = min(TJ, n_j - t * TJ);
                unsigned next = 0u;
                if (t + 1 < ntile) {
                    next = load_tile(t + 1);
                    cp_async_wait<1>();
                } else {
                    cp_async_wait<0>();
                }
                shift_tile(t, codes);
                codes = next;
                __syncthreads();  // tile t in shared memory for every thread
                const float *jx = reinterpret_cast<const float *>(jbuf + (t & 1) * 4 * TJ);
                const unsigned *jidt = jbuf + (t & 1) * 4 * TJ + 3 * TJ;

                // Bins every slot of this warp's lanes, two slots per round
                // so that their shared-memory load chains overlap.
                auto warp_flush = [&]() {
                    const int maxc = __reduce_max_sync(0xffffffffu, (unsigned)cnt);
                    for (int q0 = 0; q0 < maxc; q0 += FLUSH_ILP) {
                        uint2 e[FLUSH_ILP];
                        bool v[FLUSH_ILP];
#pragma unroll
                        for (int u = 0; u < FLUSH_ILP; ++u) {
                            v[u] = q0 + u < cnt;
                            // rows < SLOTS (q0 even, SLOTS even): load, then select
                            const uint2 g = my_slots[(q0 + u) * NT];
                            e[u] = make_uint2(v[u] ? g.x : 0x7f800000u, v[u] ? g.y : 0u);
                        }
                        int ch[FLUSH_ILP], bi[FLUSH_ILP], ia[FLUSH_ILP], ja[FLUSH_ILP];
                        bool ok[FLUSH_ILP], need[FLUSH_ILP];
#pragma unroll
                        for (int u = 0; u < FLUSH_ILP; ++u) {
                            const float d2 = __uint_as_float(e[u].x);
                            const int r = e[u].y & 3;  // R <= 4
                            const int jj = (e[u].y >> 2) & 0x1fff;
                            const unsigned iv = s_iv[r][tid];  // written by this thread
                            const int t_i = (int)(iv >> 24);
                            const unsigned jv = jidt[jj];
                            ia[u] = (int)(iv & 0xffffffu);
                            ja[u] = (int)(jv & 0xffffffu);
                            ch[u] = chtab[t_i * P.ntypes + (int)(jv >> 24)] +
                                    (ia[u] == ja[u] ? half : 0);
                            const int b_ = __float2int_rd(
                                __fmul_rn(__fsub_rn(sqrt_guess(d2), P.rmin_f), P.inv_dr_f));
                            bi[u] = min(max(b_, 0), P.nbin - 1);
                            const float2 w = win[bi[u]];
                            const bool test = v[u] && d2 >= P.lo_f;
                            const bool inw = d2 >= w.x && d2 <= w.y;
                            ok[u] = test && inw;
                            need[u] = test && !inw;
                        }
#pragma unroll
                        for (int u = 0; u < FLUSH_ILP; ++u)
                            red_shared_add1_if(smem_u32(hist + ch[u] * P.nbin + bi[u]),
                                               ok[u] && GOFR_CHECK(ch[u] >= 0 && ch[u] < P.nch &&
                                                                       bi[u] >= 0 && bi[u] < P.nbin,
                                                                   P.err));
                        // FP64 rechecks are rare: one warp-uniform branch
                        // around them
                        bool any_need = false;
#pragma unroll
                        for (int u = 0; u < FLUSH_ILP; ++u) any_need |= need[u];
                        if (__any_sync(0xffffffffu, any_need)) {
#pragma unroll
                            for (int u = 0; u < FLUSH_ILP; ++u) {
                                if (!need[u]) continue;
                                ++n_rech;
                                const int slot = atomicAdd(&rqn, 1);
                                if (slot < QCAP) {
                                    rq[slot] = make_uint4((unsigned)ia[u], (unsigned)ja[u],
                                                          (unsigned)ch[u], 0u);
                                } else {
                                    const double *xi64 = P.pos64 + (fo * P.N + ia[u]) * 3;
                                    const double *xj64 = P.pos64 + (fl * P.N + ja[u]) * 3;
                                    const double d2d =
                                        ref_d2<false>(xi64[0], xi64[1], xi64[2], xj64[0], xj64[1],
                                                      xj64[2], P.box64 + fo * 9, P.err);
                                    const int bb =
                                        ref_bin(d2d, P.rmin, P.dr, P.rmin2, P.rmax2, P.nbin);
                                    if (bb >= 0) atomicAdd(hist + ch[u] * P.nbin + bb, 1u);
                                }
                            }
                        }
                    }
                    n_cand += cnt;
                    cnt = 0;
                };

                for (int jj = 0; jj < tj; jj += 4) {
                    const float4 X = *reinterpret_cast<const float4 *>(jx + jj);
                    const float4 Y = *reinterpret_cast<const float4 *>(jx + TJ + jj);
                    const float4 Z = *reinterpret_cast<const float4 *>(jx + 2 * TJ + jj);
                    const f2 xa = f2pk(X.x, X.y), xb = f2pk(X.z, X.w);
                    const f2 ya = f2pk(Y.x, Y.y), yb = f2pk(Y.z, Y.w);
                    const f2 za = f2pk(Z.x, Z.y), zb = f2pk(Z.z, Z.w);
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const f2 da = pair2s(xi[r], yi[r], zi[r], xa, ya, za);
                        const f2 db = pair2s(xi[r], yi[r], zi[r], xb, yb, zb);
                        float d0, d1, d2v, d3;
                        f2up(da, d0, d1);
                        f2up(db, d2v, d3);
                        const unsigned m0 = (unsigned)((jj << 2) | r);
                        if (d0 <= hi_f) { my_slots[cnt * NT] = make_uint2(__float_as_uint(d0), m0); ++cnt; }
                        if (d1 <= hi_f) { my_slots[cnt * NT] = make_uint2(__float_as_uint(d1), m0 + 4u); ++cnt; }
                        if (d2v <= hi_f) { my_slots[cnt * NT] = make_uint2(__float_as_uint(d2v), m0 + 8u); ++cnt; }
                        if (d3 <= hi_f) { my_slots[cnt * NT] = make_uint2(__float_as_uint(d3), m0 + 12u); ++cnt; }
                        if (!GOFR_CHECK(cnt <= SLOTS, P.err)) cnt = SLOTS;
                        if (__any_sync(0xffffffffu, cnt > SLOTS - 4)) warp_flush();
                    }
                }
                if (__any_sync(0xffffffffu, cnt > 0)) warp_flush();
                __syncthreads();  // every thread done with buffer t & 1
                // FP64 recheck queue more than half full: drain it now, all
                // threads together (the same decision in every thread), so that
                // it rarely fills and a flush rarely recomputes a pair itself
                if (rqn > QCAP / 2) {
                    const int nq = min(rqn, QCAP);
                    for (int q = tid; q < nq; q += NT) {
                        const uint4 e = rq[q];
                        const double *xi64 = P.pos64 + (fo * P.N + (int)e.x) * 3;
                        const double *xj64 = P.pos64 + (fl * P.N + (int)e.y) * 3;
                        const double d2d = ref_d2<false>(xi64[0], xi64[1], xi64[2], xj64[0],
                                                         xj64[1], xj64[2], P.box64 + fo * 9, P.err);
                        const int bb = ref_bin(d2d, P.rmin, P.dr, P.rmin2, P.rmax2, P.nbin);
                        if (bb >= 0) atomicAdd(hist + (int)e.z * P.nbin + bb, 1u);
                    }
                    __syncthreads();
                    if (tid == 0) rqn = 0;
                    __syncthreads();
                }
            }
        }
        // end of item: FP64 recheck queue of this item's frames, all threads together
        __syncthreads();
        const int nq = min(rqn, QCAP);
        for (int q = tid; q < nq; q += NT) {
            const uint4 e = rq[q];
            const double *xi64 = P.pos64 + (fo * P.N + (int)e.x) * 3;
            const double *xj64 = P.pos64 + (fl * P.N + (int)e.y) * 3;
            const double d2d = ref_d2<false>(xi64[0], xi64[1], xi64[2], xj64[0], xj64[1], xj64[2],
                                             P.box64 + fo * 9, P.err);
            const int bb = ref_bin(d2d, P.rmin, P.dr, P.rmin2, P.rmax2, P.nbin);
            if (bb >= 0) atomicAdd(hist + (int)e.z * P.nbin + bb, 1u);
        }
        __syncthreads();
        if (tid == 0) rqn = 0;
    }
    if (cur_lag >= 0) {
        __syncthreads();
        flush_hist();
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_cand += __shfl_xor_sync(0xffffffffu, n_cand, o);
        n_rech += __shfl_xor_sync(0xffffffffu, n_rech, o);
        n_eval += __shfl_xor_sync(0xffffffffu, n_eval, o);
    }
    if ((tid & 31) == 0) {
        if (n_cand) atomicAdd(P.stats + ST_CANDIDATES, n_cand);
        if (n_rech) atomicAdd(P.stats + ST_RECHECKS, n_rech);
        if (n_eval) atomicAdd(P.stats + ST_EVALUATED, n_eval);
    }
}

}  // namespace cells

int cell_smem_bytes(int nch, int nbin, int ntypes)
{
    using namespace cells;
    size_t b = (size_t)2 * 4 * TJ * 4 + (size_t)SLOTS * NT * 8 + (size_t)QCAP * 16 +
               (size_t)nbin * 8 + (size_t)nch * nbin * 4 + (size_t)ntypes * ntypes * 2;
    return (int)((b + 127) / 128 * 128);
}

int cell_block_atoms(int r) { return cells::NT * r; }
int cell_max_ranges() { return cells::MAXR; }

int launch_cell_build(const double *pos64, const unsigned char *types8, size_t T, size_t N,
                      const double *box_internal, const double *centre, const int *nc, bool tric,
                      int *cell_of, int *rank_of, int *count, int *start, float *spos,
                      unsigned *sidt, cudaStream_t s)
{
    using namespace cells;
    if (tric && (spos || sidt)) return -1;  // the block kernel's frames are orthorhombic
    const int ncell = nc[0] * nc[1] * nc[2];
    if (cudaMemsetAsync(count, 0, T * (size_t)(ncell + 1) * sizeof(int), s) != cudaSuccess)
        return -1;
    const size_t NP = padded_natoms(N);
    // padding of the sorted frames: NaN coordinates (never read as atoms)
    if (spos && cudaMemsetAsync(spos, 0xff, T * 3 * NP * sizeof(float), s) != cudaSuccess)
        return -1;
    const size_t total = T * N;
    int blocks = (int)((total + NT - 1) / NT);
    if (blocks > 152 * 16) blocks = 152 * 16;
    const double Lx = 2.0 * box_internal[3], Ly = 2.0 * box_internal[4], Lz = 2.0 * box_internal[5];
    k_cell_assign<<<blocks, NT, 0, s>>>(pos64, T, N, box_internal[0], box_internal[1],
                                        box_internal[2], Lx, Ly, Lz, box_internal[6],
                                        box_internal[7], box_internal[8], tric ? 1 : 0, nc[0],
                                        nc[1], nc[2], cell_of, rank_of, count);
    k_cell_scan<<<(unsigned)T, NT, 0, s>>>(count, start, ncell);
    if (spos && sidt)
        k_cell_scatter<<<blocks, NT, 0, s>>>(pos64, types8, T, N, NP, ncell, box_internal[0],
                                             box_internal[1], box_internal[2], Lx, Ly, Lz,
                                             centre[0], centre[1], centre[2], cell_of, rank_of,
                                             start, spos, sidt);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int R, bool MULTI>
static int launch_cell_r(const CellLaunch &C, const CellLaunch *d_cells, const long long *d_end,
                         int nmem, long long total, int max_nbin, int max_nch, int max_ntypes,
                         int num_sms, cudaStream_t s)
{
    using namespace cells;
    const int smem = cell_smem_bytes(max_nch, max_nbin, max_ntypes);
    if (cudaFuncSetAttribute(k_pairs_cell<R, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pairs_cell<R, MULTI>, NT, smem) !=
        cudaSuccess)
        return -1;
    if (per_sm < 1) return -2;
    long long grid = (long long)num_sms * per_sm;
    if (grid > total) grid = total;
    k_pairs_cell<R, MULTI><<<(unsigned)grid, NT, smem, s>>>(C, d_cells, d_end, nmem, max_nbin,
                                                             max_nch * max_nbin);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_cell_pairs(const CellLaunch &C, int num_sms, cudaStream_t s)
{
    const long long total = C.pair.n_items;
    if (total <= 0) return 0;
    const int nb = C.pair.nbin, nc = C.pair.nch, nt = C.pair.ntypes;
    switch (C.r) {
    case 2: return launch_cell_r<2, false>(C, nullptr, nullptr, 1, total, nb, nc, nt, num_sms, s);
    case 3: return launch_cell_r<3, false>(C, nullptr, nullptr, 1, total, nb, nc, nt, num_sms, s);
    case 4: return launch_cell_r<4, false>(C, nullptr, nullptr, 1, total, nb, nc, nt, num_sms, s);
    default: return -3;
    }
}

template <int R>
static int prepare_multi_r(int smem, int num_sms, long long total, int *grid)
{
    using namespace cells;
    if (cudaFuncSetAttribute(k_pairs_cell<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pairs_cell<R, true>, NT, smem) !=
        cudaSuccess)
        return -1;
    if (per_sm < 1) return -2;
    long long g = (long long)num_sms * per_sm;
    if (g > total) g = total;
    *grid = (int)g;
    return 0;
}

int prepare_cell_pairs_multi(int r, int max_nbin, int max_nch, int max_ntypes, int num_sms,
                             long long total, int *grid)
{
    const int smem = cell_smem_bytes(max_nch, max_nbin, max_ntypes);
    switch (r) {
    case 2: return prepare_multi_r<2>(smem, num_sms, total, grid);
    case 3: return prepare_multi_r<3>(smem, num_sms, total, grid);
    case 4: return prepare_multi_r<4>(smem, num_sms, total, grid);
    default: return -3;
    }
}

int launch_cell_pairs_multi(const CellLaunch *d_cells, const long long *d_end, int nmem,
                            int r, int max_nbin, int max_nch, int max_ntypes, int grid,
                            cudaStream_t s)
{
    using namespace cells;
    if (grid <= 0 || nmem <= 0) return 0;
    const int smem = cell_smem_bytes(max_nch, max_nbin, max_ntypes);
    const CellLaunch none{};
    switch (r) {
    case 2: k_pairs_cell<2, true><<<grid, NT, smem, s>>>(none, d_cells, d_end, nmem, max_nbin, max_nch * max_nbin); break;
    case 3: k_pairs_cell<3, true><<<grid, NT, smem, s>>>(none, d_cells, d_end, nmem, max_nbin, max_nch * max_nbin); break;
    case 4: k_pairs_cell<4, true><<<grid, NT, smem, s>>>(none, d_cells, d_end, nmem, max_nbin, max_nch * max_nbin); break;
    default: return -3;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gofr
