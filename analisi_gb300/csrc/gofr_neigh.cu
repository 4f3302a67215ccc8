// Neighbour lists of one resident frame (the reference's
// Neighbours<T,double>::update_neigh, lib/src/neighbour.cpp:9-79).
//
// The reference visits the pairs i < j once and appends each pair within
// either type's cutoff to both atoms' lists, so every list ends up in
// ascending neighbour index.  Here one warp builds one atom's lists: its lanes
// take 32 consecutive candidates at a time, compute the reference's FP64
// minimum-image vector for the ordered pair (lower index first, negated for
// the higher-index atom, as the reference stores -x), and the counted entries
// of each neighbour type are placed by a ballot prefix, which keeps the
// ascending order.  Where the all-pairs kernel's FP32 bound certifies it, an
// FP32 minimum-image d2 first discards the pairs beyond every cutoff; the
// remaining candidates are queued in shared memory (ascending) and their FP64
// arithmetic runs 32 at a time, one per lane, so the slow FP64 pipe works only
// on full warps of near pairs.  Overflow follows the reference's rule exactly: a pair
// (i < j) within either cutoff is an error when, at that point of the
// reference's loop, i's list of j's type or j's list of i's type is full;
// with full[a][k] = the neighbour index that filled a's list of type k, that
// is full[i][t_j] < j or full[j][t_i] < i, checked by a second pass (only
// when some list is full) that keeps the first such pair in loop order.  The
// optional sort by distance is a stable insertion sort per list.
#include <cstdint>
#include <cuda_runtime.h>

#include "gofr_device.cuh"
#include "gofr_internal.h"

namespace gofr {
namespace neigh {

constexpr int NT = 256;
constexpr int WARPS = NT / 32;

// x = minimum image of x_i - x_j (i < j), d2 as the reference
template <bool TRI>
__device__ __forceinline__ double pair_vec(const NeighLaunch &L, const double *frame,
                                           const double *box, int i, int j, double x[3])
{
    const double *pi = frame + (size_t)i * 3, *pj = frame + (size_t)j * 3;
    x[0] = __dsub_rn(pi[0], pj[0]);
    x[1] = __dsub_rn(pi[1], pj[1]);
    x[2] = __dsub_rn(pi[2], pj[2]);
    ref_min_image<TRI>(x[0], x[1], x[2], box, L.err);
    double s = __dmul_rn(x[0], x[0]);
    s = __dadd_rn(s, __dmul_rn(x[1], x[1]));
    s = __dadd_rn(s, __dmul_rn(x[2], x[2]));
    return s;
}

// FP32 minimum-image d2 of one pair with exactly the all-pairs kernel's
// operations (gofr_kernels.cu pair2<TRI, false>, one lane), so that kernel's
// certified bound applies: d2_f32 > hi_f implies the reference's d2 exceeds
// every cutoff.
template <bool TRI>
__device__ __forceinline__ float pair_f32(const NeighLaunch &L, int a, int b)
{
    const float MAG = 12582912.0f;
    const float *f = L.pos32 + L.timestep * 3 * L.NP;
    const Box32 bx = L.box32[L.timestep];
    float dx = __fsub_rn(f[a], f[b]);
    float dy = __fsub_rn(f[L.NP + a], f[L.NP + b]);
    float dz = __fsub_rn(f[2 * L.NP + a], f[2 * L.NP + b]);
    if (TRI) {
        const float kz = __fsub_rn(__fmaf_rn(dz, bx.invL[2], MAG), MAG);
        dz = __fmaf_rn(kz, -bx.L[2], dz);
        dy = __fmaf_rn(kz, -bx.tilt[2], dy);
        dx = __fmaf_rn(kz, -bx.tilt[1], dx);
        const float ky = __fsub_rn(__fmaf_rn(dy, bx.invL[1], MAG), MAG);
        dy = __fmaf_rn(ky, -bx.L[1], dy);
        dx = __fmaf_rn(ky, -bx.tilt[0], dx);
        const float kx = __fsub_rn(__fmaf_rn(dx, bx.invL[0], MAG), MAG);
        dx = __fmaf_rn(kx, -bx.L[0], dx);
    } else {
        const float kx = __fsub_rn(__fmaf_rn(dx, bx.invL[0], MAG), MAG);
        const float ky = __fsub_rn(__fmaf_rn(dy, bx.invL[1], MAG), MAG);
        const float kz = __fsub_rn(__fmaf_rn(dz, bx.invL[2], MAG), MAG);
        dx = __fmaf_rn(kx, -bx.L[0], dx);
        dy = __fmaf_rn(ky, -bx.L[1], dy);
        dz = __fmaf_rn(kz, -bx.L[2], dz);
    }
    float d2 = __fmul_rn(dx, dx);
    d2 = __fmaf_rn(dy, dy, d2);
    d2 = __fmaf_rn(dz, dz, d2);
    return d2;
}

// FP64 arithmetic and placement of the n (<= 32) candidates src[0..n) of
// atom a, one per lane, in ascending order: the counted entries of each
// neighbour type go to the list at the running count cnt[k] (ballot prefix),
// and full[a][k] records the neighbour that fills a list.
template <bool TRI>
__device__ __forceinline__ void place(const NeighLaunch &L, const double *frame, const double *box,
                                      int a, const int *src, int n, unsigned long long *cnt)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const bool have = lane < n;
    const int b = have ? src[lane] : 0;
    int tb = 0;
    double x[3] = {0.0, 0.0, 0.0}, d2 = 0.0;
    bool counted = false;
    if (have) {
        tb = L.types[b];
        const int i = a < b ? a : b, j = a < b ? b : a;
        d2 = pair_vec<TRI>(L, frame, box, i, j, x);
        if (a > b) { x[0] = -x[0]; x[1] = -x[1]; x[2] = -x[2]; }
        counted = d2 <= L.cut2[tb];
    }
    for (int k = 0; k < L.ntypes; ++k) {
        const unsigned m = __ballot_sync(0xffffffffu, counted && tb == k);
        if (!m) continue;
        const unsigned long long base = cnt[k];
        const unsigned long long nk = L.nneigh[k];
        if (counted && tb == k) {
            const unsigned long long pos = base + __popc(m & lt);
            if (pos < nk) {
                L.list[L.loff[k] + (size_t)a * (nk + 1) + 1 + pos] = (unsigned long long)b;
                double *r = L.rpos + L.roff[k] + ((size_t)a * nk + pos) * 4;
                r[0] = __dsqrt_rn(d2);
                r[1] = x[0];
                r[2] = x[1];
                r[3] = x[2];
            }
            if (pos + 1 == nk) L.full[(size_t)a * L.ntypes + k] = b;
        }
        __syncwarp();
        if (lane == 0) cnt[k] = base + __popc(m);
        __syncwarp();
    }
}

template <bool TRI>
__global__ void __launch_bounds__(NT) k_neigh_build(const NeighLaunch L)
{
    __shared__ unsigned long long cnt[WARPS][NEIGH_MAXT];
    __shared__ int cq[WARPS][64];  // candidates of this warp's atom, ascending
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const double *frame = L.pos64 + (size_t)L.timestep * L.N * 3;
    const double *box = L.box64 + (size_t)L.timestep * 9;
    const unsigned lt = (1u << lane) - 1u;
    for (long long a0 = (long long)blockIdx.x * WARPS; a0 < L.N; a0 += (long long)gridDim.x * WARPS) {
        const int a = (int)(a0 + w);
        if (a >= L.N) continue;  // warp-uniform
        for (int k = lane; k < L.ntypes; k += 32) {
            cnt[w][k] = 0ull;
            // a list of capacity 0 is full before its first neighbour
            L.full[(size_t)a * L.ntypes + k] = L.nneigh[k] == 0 ? -1 : L.N;
        }
        __syncwarp();
        int qn = 0;  // queued candidates (warp-uniform)
        for (int b0 = 0; b0 < L.N; b0 += 32) {
            const int b = b0 + lane;
            bool cand = b < L.N && b != a;
            if (cand && L.prefilter) cand = pair_f32<TRI>(L, a, b) <= L.hi_f;
            const unsigned m = __ballot_sync(0xffffffffu, cand);
            if (!m) continue;
            if (cand) cq[w][qn + __popc(m & lt)] = b;
            qn += __popc(m);
            __syncwarp();
            if (qn >= 32) {
                place<TRI>(L, frame, box, a, cq[w], 32, cnt[w]);
                const int rest = qn - 32;
                const int v = lane < rest ? cq[w][32 + lane] : 0;
                __syncwarp();
                if (lane < rest) cq[w][lane] = v;
                __syncwarp();
                qn = rest;
            }
        }
        if (qn > 0) place<TRI>(L, frame, box, a, cq[w], qn, cnt[w]);
        for (int k = lane; k < L.ntypes; k += 32) {
            const unsigned long long c = cnt[w][k], nk = L.nneigh[k];
            L.list[L.loff[k] + (size_t)a * (nk + 1)] = c < nk ? c : nk;
            if (c >= nk) atomicOr(L.flags, 1u);  // some list is full: run the check
        }
        __syncwarp();
    }
}

// Cell-list form (orthorhombic boxes): the frame's atoms sorted by cells of
// edge >= the largest cutoff, at least 3 per axis, so every pair within a
// cutoff lies in neighbouring cells.  A warp takes the atom of one sorted
// slot, gathers the atoms of the 27 cells around its cell through the FP32
// prefilter, sorts the survivors by index (the reference's list order) and
// places them as the all-pairs form does.  A neighbourhood with more than
// CQCAP survivors sets flags bit 1 and the host runs the all-pairs form.
constexpr int CQCAP = 256;

__global__ void __launch_bounds__(NT) k_neigh_build_cells(const NeighLaunch L)
{
    __shared__ unsigned long long cnt[WARPS][NEIGH_MAXT];
    __shared__ int cq[WARPS][CQCAP];  // survivors in cell order
    __shared__ int cs[WARPS][CQCAP];  // the same, ascending
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const double *frame = L.pos64 + (size_t)L.timestep * L.N * 3;
    const double *box = L.box64 + (size_t)L.timestep * 9;
    const unsigned lt = (1u << lane) - 1u;
    const int nx = L.nc[0], ny = L.nc[1], nz = L.nc[2];
    const int ncell = nx * ny * nz;
    for (long long s0 = (long long)blockIdx.x * WARPS; s0 < L.N; s0 += (long long)gridDim.x * WARPS) {
        const int s = (int)(s0 + w);
        if (s >= L.N) continue;  // warp-uniform
        const int a = (int)(L.csidt[s] & 0xffffffu);
        // the cell of slot s: the last cell whose first slot is <= s
        int lo = 0, hi = ncell - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (L.cstart[mid] <= s) lo = mid;
            else hi = mid - 1;
        }
        const int cx = lo % nx, cy = (lo / nx) % ny, cz = lo / (nx * ny);
        for (int k = lane; k < L.ntypes; k += 32) {
            cnt[w][k] = 0ull;
            L.full[(size_t)a * L.ntypes + k] = L.nneigh[k] == 0 ? -1 : L.N;
        }
        // lane k < 27 takes neighbour cell k: its first slot and atom count
        int beg = 0, num = 0;
        if (lane < 27) {
            const int ux = (cx + lane % 3 - 1 + nx) % nx;
            const int uy = (cy + (lane / 3) % 3 - 1 + ny) % ny;
            const int uz = (cz + lane / 9 - 1 + nz) % nz;
            const int cc = (uz * ny + uy) * nx + ux;
            beg = L.cstart[cc];
            num = L.cstart[cc + 1] - beg;
        }
        int incl = num;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int excl = incl - num;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int qn = 0;  // survivors (warp-uniform)
        bool over = false;
        for (int f0 = 0; f0 < total; f0 += 32) {
            const int f = f0 + lane;
            // the neighbour cell holding flat index f: the last lane with excl <= f
            int src = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int e = __shfl_sync(0xffffffffu, excl, src + step);
                if (e <= f) src += step;
            }
            const int sb = __shfl_sync(0xffffffffu, beg, src) + f -
                           __shfl_sync(0xffffffffu, excl, src);
            bool cand = false;
            int b = 0;
            if (f < total) {
                b = (int)(L.csidt[sb] & 0xffffffu);
                cand = b != a && pair_f32<false>(L, a, b) <= L.hi_f;
            }
            const unsigned m = __ballot_sync(0xffffffffu, cand);
            if (qn + __popc(m) > CQCAP) {
                over = true;
                break;
            }
            if (cand) cq[w][qn + __popc(m & lt)] = b;
            qn += __popc(m);
        }
        if (over) {
            if (lane == 0) atomicOr(L.flags, 2u);
            continue;
        }
        __syncwarp();
        // ascending order: the rank of each survivor among the (distinct) indices
        for (int k = lane; k < qn; k += 32) {
            const int v = cq[w][k];
            int rank = 0;
            for (int q = 0; q < qn; ++q) rank += cq[w][q] < v ? 1 : 0;
            cs[w][rank] = v;
        }
        __syncwarp();
        for (int p0 = 0; p0 < qn; p0 += 32)
            place<false>(L, frame, box, a, cs[w] + p0, min(32, qn - p0), cnt[w]);
        for (int k = lane; k < L.ntypes; k += 32) {
            const unsigned long long c = cnt[w][k], nk = L.nneigh[k];
            L.list[L.loff[k] + (size_t)a * (nk + 1)] = c < nk ? c : nk;
            if (c >= nk) atomicOr(L.flags, 1u);  // some list is full: run the check
        }
        __syncwarp();
    }
}

// first pair (i < j) in the reference's loop order that finds a full list
template <bool TRI>
__global__ void __launch_bounds__(NT) k_neigh_check(const NeighLaunch L)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const double *frame = L.pos64 + (size_t)L.timestep * L.N * 3;
    const double *box = L.box64 + (size_t)L.timestep * 9;
    for (long long a0 = (long long)blockIdx.x * WARPS; a0 < L.N; a0 += (long long)gridDim.x * WARPS) {
        const int i = (int)(a0 + w);
        if (i >= L.N) continue;
        const int ti = L.types[i];
        for (int j = i + 1 + lane; j < L.N; j += 32) {
            if (L.prefilter && !(pair_f32<TRI>(L, i, j) <= L.hi_f)) continue;
            const int tj = L.types[j];
            double x[3];
            const double d2 = pair_vec<TRI>(L, frame, box, i, j, x);
            if (!(d2 <= L.cut2[tj] || d2 <= L.cut2[ti])) continue;
            if (L.full[(size_t)i * L.ntypes + tj] < j || L.full[(size_t)j * L.ntypes + ti] < i)
                atomicMin(L.first_err, (unsigned long long)i * (unsigned long long)L.N + j);
        }
    }
}

// The check in the cell-list form: the same pairs (i < j within either
// cutoff) come from the 27 cells around i's cell, one warp per first atom;
// the minimum over them is order-independent.
__global__ void __launch_bounds__(NT) k_neigh_check_cells(const NeighLaunch L)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const double *frame = L.pos64 + (size_t)L.timestep * L.N * 3;
    const double *box = L.box64 + (size_t)L.timestep * 9;
    const int nx = L.nc[0], ny = L.nc[1], nz = L.nc[2];
    const int ncell = nx * ny * nz;
    for (long long s0 = (long long)blockIdx.x * WARPS; s0 < L.N; s0 += (long long)gridDim.x * WARPS) {
        const int s = (int)(s0 + w);
        if (s >= L.N) continue;  // warp-uniform
        const int i = (int)(L.csidt[s] & 0xffffffu);
        const int ti = L.types[i];
        int lo = 0, hi = ncell - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (L.cstart[mid] <= s) lo = mid;
            else hi = mid - 1;
        }
        const int cx = lo % nx, cy = (lo / nx) % ny, cz = lo / (nx * ny);
        for (int c = 0; c < 27; ++c) {
            const int ux = (cx + c % 3 - 1 + nx) % nx;
            const int uy = (cy + (c / 3) % 3 - 1 + ny) % ny;
            const int uz = (cz + c / 9 - 1 + nz) % nz;
            const int cc = (uz * ny + uy) * nx + ux;
            const int beg = L.cstart[cc], end = L.cstart[cc + 1];
            for (int q = beg + lane; q < end; q += 32) {
                const int j = (int)(L.csidt[q] & 0xffffffu);
                if (j <= i || !(pair_f32<false>(L, i, j) <= L.hi_f)) continue;
                const int tj = L.types[j];
                double x[3];
                const double d2 = pair_vec<false>(L, frame, box, i, j, x);
                if (!(d2 <= L.cut2[tj] || d2 <= L.cut2[ti])) continue;
                if (L.full[(size_t)i * L.ntypes + tj] < j || L.full[(size_t)j * L.ntypes + ti] < i)
                    atomicMin(L.first_err, (unsigned long long)i * (unsigned long long)L.N + j);
            }
        }
    }
}

// Every list sorted by distance, stably (equal distances keep their index
// order), as the reference's sort.  One warp per list: lane q holds entries
// q, q + 32, ... (up to SORTC per lane) in registers and their distances in
// shared memory, ranks each one against the whole list (rank = entries with
// a smaller distance, or an equal one earlier), then writes it at its rank.
// A longer list is insertion-sorted by the warp's first lane.
constexpr int SORTC = 4;

__global__ void __launch_bounds__(NT) k_neigh_sort(const NeighLaunch L)
{
    __shared__ double sd[WARPS][32 * SORTC];
    const int lane = threadIdx.x & 31;
    double *const d = sd[threadIdx.x >> 5];
    const long long n_lists = (long long)L.N * L.ntypes;
    const long long nwarps = (long long)gridDim.x * WARPS;
    for (long long g = (long long)blockIdx.x * WARPS + (threadIdx.x >> 5); g < n_lists;
         g += nwarps) {
        const int k = (int)(g / L.N), a = (int)(g - (long long)k * L.N);
        const unsigned long long nk = L.nneigh[k];
        unsigned long long *l = L.list + L.loff[k] + (size_t)a * (nk + 1);
        double *r = L.rpos + L.roff[k] + (size_t)a * nk * 4;
        const int n = (int)l[0];
        if (n <= 1) continue;  // warp-uniform
        if (n > 32 * SORTC) {
            if (lane == 0) {
                for (int s = 1; s < n; ++s) {
                    const double e0 = r[4 * s], e1 = r[4 * s + 1], e2 = r[4 * s + 2],
                                 e3 = r[4 * s + 3];
                    const unsigned long long id = l[1 + s];
                    int q = s;
                    while (q > 0 && e0 < r[4 * (q - 1)]) {
                        r[4 * q] = r[4 * (q - 1)];
                        r[4 * q + 1] = r[4 * (q - 1) + 1];
                        r[4 * q + 2] = r[4 * (q - 1) + 2];
                        r[4 * q + 3] = r[4 * (q - 1) + 3];
                        l[1 + q] = l[q];
                        --q;
                    }
                    r[4 * q] = e0;
                    r[4 * q + 1] = e1;
                    r[4 * q + 2] = e2;
                    r[4 * q + 3] = e3;
                    l[1 + q] = id;
                }
            }
            __syncwarp();
            continue;
        }
        double e0[SORTC], e1[SORTC], e2[SORTC], e3[SORTC];
        unsigned long long id[SORTC];
        int rank[SORTC];
#pragma unroll
        for (int c = 0; c < SORTC; ++c) {
            const int q = lane + 32 * c;
            rank[c] = -1;
            if (q < n) {
                e0[c] = r[4 * q];
                e1[c] = r[4 * q + 1];
                e2[c] = r[4 * q + 2];
                e3[c] = r[4 * q + 3];
                id[c] = l[1 + q];
                rank[c] = 0;
                d[q] = e0[c];
            }
        }
        __syncwarp();
        for (int m = 0; m < n; ++m) {
            const double v = d[m];
#pragma unroll
            for (int c = 0; c < SORTC; ++c) {
                const int q = lane + 32 * c;
                if (q < n) rank[c] += (v < e0[c] || (v == e0[c] && m < q)) ? 1 : 0;
            }
        }
        __syncwarp();  // every entry read before any is moved
#pragma unroll
        for (int c = 0; c < SORTC; ++c) {
            if (rank[c] >= 0) {
                const int q = rank[c];
                r[4 * q] = e0[c];
                r[4 * q + 1] = e1[c];
                r[4 * q + 2] = e2[c];
                r[4 * q + 3] = e3[c];
                l[1 + q] = id[c];
            }
        }
        __syncwarp();
    }
}

}  // namespace neigh

int launch_neigh_build(const NeighLaunch &L, int num_sms, cudaStream_t s)
{
    using namespace neigh;
    long long grid = (L.N + WARPS - 1) / WARPS;
    if (grid > (long long)num_sms * 16) grid = (long long)num_sms * 16;
    if (grid < 1) return 0;
    if (L.cells && !L.tric && L.prefilter) k_neigh_build_cells<<<(unsigned)grid, NT, 0, s>>>(L);
    else if (L.tric) k_neigh_build<true><<<(unsigned)grid, NT, 0, s>>>(L);
    else k_neigh_build<false><<<(unsigned)grid, NT, 0, s>>>(L);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_neigh_check(const NeighLaunch &L, int num_sms, cudaStream_t s)
{
    using namespace neigh;
    long long grid = (L.N + WARPS - 1) / WARPS;
    if (grid > (long long)num_sms * 16) grid = (long long)num_sms * 16;
    if (grid < 1) return 0;
    if (L.cells && !L.tric && L.prefilter) k_neigh_check_cells<<<(unsigned)grid, NT, 0, s>>>(L);
    else if (L.tric) k_neigh_check<true><<<(unsigned)grid, NT, 0, s>>>(L);
    else k_neigh_check<false><<<(unsigned)grid, NT, 0, s>>>(L);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_neigh_sort(const NeighLaunch &L, int num_sms, cudaStream_t s)
{
    using namespace neigh;
    long long n = (long long)L.N * L.ntypes;  // lists, one warp each
    long long grid = (n + WARPS - 1) / WARPS;
    if (grid > (long long)num_sms * 16) grid = (long long)num_sms * 16;
    if (grid < 1) return 0;
    k_neigh_sort<<<(unsigned)grid, NT, 0, s>>>(L);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gofr
