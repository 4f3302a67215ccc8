// Gofrt pair/histogram kernels for GB300 (sm_103a).
//
// Replaces the reference's hot loop Gofrt::calc_single_th
// (lib/src/gofrt.cpp:96-122, with the inlined geometry of
// lib/include/basetrajectory.h:181-268) and its fork/join driver
// (lib/include/calculatemultithread.h:106-162).
//
// Work decomposition: one launch covers every (lag, first-atom tile, origin)
// item of a Gofrt::calculate.  A persistent grid of CTAs takes contiguous,
// lag-major ranges of items, so consecutive items of a CTA share the lag and
// its shared-memory histogram [nch][nbin] is flushed to the global u64 counts
// only when the lag changes (or before a u32 bin could overflow).  Inside an
// item, each thread holds R first atoms (frame `origin`) in registers and the
// CTA streams the second atoms (frame `origin+lag`) through shared memory in
// tiles of TJ atoms, double buffered with 1-D TMA bulk copies completed on
// mbarriers.
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "gofr_device.cuh"
#include "gofr_internal.h"

namespace gofr {

constexpr int NT = 256;      // threads per CTA
constexpr int R32 = 2;       // first atoms per thread, FP32 kernel
constexpr int TI32 = NT * R32;
constexpr int TJ32 = 1024;   // second atoms per shared-memory tile (16 KB of float4)
constexpr int R64 = 2;
constexpr int TI64 = NT * R64;
constexpr int TJ64 = 512;

// Items per flush so that no u32 shared bin can overflow: one item adds at
// most TI*N hits to one bin.
__host__ __device__ inline long long items_per_flush(int ti, int N)
{
    long long per = (1ll << 31) / ((long long)ti * (long long)(N > 0 ? N : 1));
    return per < 1 ? 1 : per;
}

__device__ __forceinline__ void decompose(long long item, const PairLaunch &P, int &lag_idx,
                                          int &itile, int &k)
{
    long long per_lag = (long long)P.n_itiles * P.n_orig;
    lag_idx = (int)(item / per_lag);
    long long rem = item - (long long)lag_idx * per_lag;
    itile = (int)(rem / P.n_orig);
    k = (int)(rem - (long long)itile * P.n_orig);
}

__device__ __forceinline__ void flush_hist(unsigned *hist, int len, unsigned long long *gout)
{
    __syncthreads();
    for (int i = threadIdx.x; i < len; i += NT) {
        unsigned v = hist[i];
        if (v) {
            atomicAdd(gout + i, (unsigned long long)v);
            hist[i] = 0u;
        }
    }
    __syncthreads();
}

__device__ __forceinline__ void add_stats(unsigned long long *stats, unsigned long long cand,
                                          unsigned long long rech)
{
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_xor_sync(0xffffffffu, cand, o);
        rech += __shfl_xor_sync(0xffffffffu, rech, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (cand) atomicAdd(stats + ST_CANDIDATES, cand);
        if (rech) atomicAdd(stats + ST_RECHECKS, rech);
    }
}

// Exact FP64 re-evaluation of one pair, exactly as the reference computes it.
template <bool TRI>
__device__ __noinline__ void recheck_pair(const double *__restrict__ pos64,
                                          const double *__restrict__ box64, long long N,
                                          long long fo, long long fl, int ia, int ja,
                                          unsigned *hist, int ch, int nbin, double rmin,
                                          double dr, double rmin2, double rmax2, unsigned *err)
{
    const double *xi = pos64 + (fo * N + ia) * 3;
    const double *xj = pos64 + (fl * N + ja) * 3;
    const double *box = box64 + fo * 9;
    double d2 = ref_d2<TRI>(xi[0], xi[1], xi[2], xj[0], xj[1], xj[2], box, err);
    int b = ref_bin(d2, rmin, dr, rmin2, rmax2, nbin);
    if (b >= 0) atomicAdd(hist + ch * nbin + b, 1u);
}

// ---------------------------------------------------------------------------
// FP32 bulk + FP64 edge recheck
// ---------------------------------------------------------------------------
//
// Per pair (orthorhombic): 3 FADD for the raw difference, per axis an FFMA
// with a 1.5*2^23 offset and an FADD that round d/L to the nearest integer k,
// an FFMA d - k*L (L rounded to FP32; its rounding is part of the bound),
// then d2 by FMUL + 2 FFMA and one compare against hi_f.
// The bound behind hi_f, lo_f and the per-bin windows is derived on the host
// (gofr_capi.cu, certify()): a pair whose FP32 d2 falls outside its bin's
// window, or (WCHK) whose wrap quotient lies within the error bound of a
// half-integer, is recomputed in FP64 by recheck_pair.
template <bool TRI, bool WCHK>
__global__ void __launch_bounds__(NT, 2) k_pairs_f32(const PairLaunch P)
{
    extern __shared__ __align__(128) unsigned char smem[];
    float4 *jbuf = reinterpret_cast<float4 *>(smem);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * TJ32 * sizeof(float4));
    int *sflag = reinterpret_cast<int *>(bars + 2);
    float2 *win = reinterpret_cast<float2 *>(smem + 2 * TJ32 * sizeof(float4) + 32);
    unsigned *hist = reinterpret_cast<unsigned *>(win + P.nbin);
    unsigned short *chtab = reinterpret_cast<unsigned short *>(hist + P.nch * P.nbin);

    const int tid = threadIdx.x;
    const int hlen = P.nch * P.nbin;
    const int half = P.nch / 2;
    for (int i = tid; i < P.nbin; i += NT) win[i] = P.win[i];
    for (int i = tid; i < hlen; i += NT) hist[i] = 0u;
    for (int i = tid; i < P.ntypes * P.ntypes; i += NT) chtab[i] = P.chtab[i];
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        *sflag = 0;
        fence_mbar_init();
    }
    __syncthreads();

    const long long per = (P.n_items + gridDim.x - 1) / gridDim.x;
    const long long it0 = (long long)blockIdx.x * per;
    const long long it1 = min(it0 + per, P.n_items);
    const long long N = P.N;
    const int nchunks = (P.N + TJ32 - 1) / TJ32;
    const long long flush_every = items_per_flush(TI32, P.N);
    const float MAGIC = 12582912.0f;  // 1.5 * 2^23

    unsigned phase0 = 0u, phase1 = 0u;
    int cur_lag = -1;
    long long since_flush = 0;
    unsigned long long n_cand = 0, n_rech = 0;
    bool failed = false;

    for (long long item = it0; item < it1 && !failed; ++item) {
        int lag_idx, itile, k;
        decompose(item, P, lag_idx, itile, k);
        if (lag_idx != cur_lag || since_flush >= flush_every) {
            if (cur_lag >= 0)
                flush_hist(hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
            cur_lag = lag_idx;
            since_flush = 0;
        }
        ++since_flush;
        const long long fo = P.primo + (long long)k * P.skip;
        const long long fl = fo + (long long)lag_idx * P.every;
        const Box32 bx = P.box32[fo];

        float xi[R32], yi[R32], zi[R32];
        int ti[R32], ia[R32];
#pragma unroll
        for (int r = 0; r < R32; ++r) {
            ia[r] = P.a0 + itile * TI32 + r * NT + tid;
            if (ia[r] < P.a1) {
                float4 p = P.pos32[fo * N + ia[r]];
                xi[r] = p.x; yi[r] = p.y; zi[r] = p.z;
                ti[r] = __float_as_int(p.w);
            } else {
                // no atom: NaN coordinates never pass d2 <= hi_f
                xi[r] = yi[r] = zi[r] = __int_as_float(0x7fc00000);
                ti[r] = 0;
            }
        }

        const float4 *jsrc = P.pos32 + fl * N;
        __syncthreads();  // previous item done with both buffers
        if (tid == 0) {
            unsigned bytes = (unsigned)(min(TJ32, P.N) * sizeof(float4));
            mbar_arrive_expect_tx(&bars[0], bytes);
            bulk_g2s(jbuf, jsrc, bytes, &bars[0]);
        }
        for (int c = 0; c < nchunks; ++c) {
            const int b = c & 1;
            if (tid == 0 && c + 1 < nchunks) {
                int nxt = min(TJ32, P.N - (c + 1) * TJ32);
                unsigned bytes = (unsigned)(nxt * sizeof(float4));
                mbar_arrive_expect_tx(&bars[b ^ 1], bytes);
                bulk_g2s(jbuf + (b ^ 1) * TJ32, jsrc + (long long)(c + 1) * TJ32, bytes,
                         &bars[b ^ 1]);
            }
            bool ok = mbar_wait_bounded(&bars[b], b ? phase1 : phase0);
            if (ok) { if (b) phase1 ^= 1u; else phase0 ^= 1u; }
            else atomicOr(sflag, 1);
            __syncthreads();
            if (*sflag) { failed = true; break; }

            const int jbase = c * TJ32;
            const int tj = min(TJ32, P.N - jbase);
            const float4 *jb = jbuf + b * TJ32;
#pragma unroll 2
            for (int jj = 0; jj < tj; ++jj) {
                const float4 pj = jb[jj];
#pragma unroll
                for (int r = 0; r < R32; ++r) {
                    float dx = __fsub_rn(xi[r], pj.x);
                    float dy = __fsub_rn(yi[r], pj.y);
                    float dz = __fsub_rn(zi[r], pj.z);
                    bool wflag = false;
                    if (TRI) {
                        float kz = __fsub_rn(__fmaf_rn(dz, bx.invL[2], MAGIC), MAGIC);
                        if (WCHK) wflag |= fabsf(__fmaf_rn(dz, bx.invL[2], -kz)) > P.wlim;
                        dz = __fmaf_rn(-kz, bx.L[2], dz);
                        dy = __fmaf_rn(-kz, bx.tilt[2], dy);
                        dx = __fmaf_rn(-kz, bx.tilt[1], dx);
                        float ky = __fsub_rn(__fmaf_rn(dy, bx.invL[1], MAGIC), MAGIC);
                        if (WCHK) wflag |= fabsf(__fmaf_rn(dy, bx.invL[1], -ky)) > P.wlim;
                        dy = __fmaf_rn(-ky, bx.L[1], dy);
                        dx = __fmaf_rn(-ky, bx.tilt[0], dx);
                        float kx = __fsub_rn(__fmaf_rn(dx, bx.invL[0], MAGIC), MAGIC);
                        if (WCHK) wflag |= fabsf(__fmaf_rn(dx, bx.invL[0], -kx)) > P.wlim;
                        dx = __fmaf_rn(-kx, bx.L[0], dx);
                    } else {
                        float kx = __fsub_rn(__fmaf_rn(dx, bx.invL[0], MAGIC), MAGIC);
                        float ky = __fsub_rn(__fmaf_rn(dy, bx.invL[1], MAGIC), MAGIC);
                        float kz = __fsub_rn(__fmaf_rn(dz, bx.invL[2], MAGIC), MAGIC);
                        if (WCHK) {
                            wflag |= fabsf(__fmaf_rn(dx, bx.invL[0], -kx)) > P.wlim;
                            wflag |= fabsf(__fmaf_rn(dy, bx.invL[1], -ky)) > P.wlim;
                            wflag |= fabsf(__fmaf_rn(dz, bx.invL[2], -kz)) > P.wlim;
                        }
                        dx = __fmaf_rn(-kx, bx.L[0], dx);
                        dy = __fmaf_rn(-ky, bx.L[1], dy);
                        dz = __fmaf_rn(-kz, bx.L[2], dz);
                    }
                    float d2 = __fmul_rn(dx, dx);
                    d2 = __fmaf_rn(dy, dy, d2);
                    d2 = __fmaf_rn(dz, dz, d2);
                    if (d2 <= P.hi_f || (WCHK && wflag)) {
                        const int ja = jbase + jj;
                        const int tj_ = __float_as_int(pj.w);
                        int ch = chtab[ti[r] * P.ntypes + tj_] + (ia[r] == ja ? half : 0);
                        ++n_cand;
                        bool need = WCHK && wflag;
                        if (!need && d2 >= P.lo_f) {
                            float rr = __fsqrt_rn(d2);
                            int bi = __float2int_rd(__fmul_rn(__fsub_rn(rr, P.rmin_f), P.inv_dr_f));
                            bi = min(max(bi, 0), P.nbin - 1);
                            const float2 w = win[bi];
                            if (d2 >= w.x && d2 <= w.y) atomicAdd(hist + ch * P.nbin + bi, 1u);
                            else need = true;
                        }
                        if (need) {
                            ++n_rech;
                            recheck_pair<TRI>(P.pos64, P.box64, N, fo, fl, ia[r], ja, hist, ch,
                                              P.nbin, P.rmin, P.dr, P.rmin2, P.rmax2, P.err);
                        }
                    }
                }
            }
            __syncthreads();  // all reads of buffer b done before it is refilled
        }
    }
    if (failed) {
        // A copy may still be in flight into either buffer (the one whose wait
        // ran out, and the prefetch of the next tile): give both a bounded
        // chance to land before the CTA exits and its shared memory is reused.
        if (tid == 0) {
            mbar_wait_bounded(&bars[0], phase0);
            mbar_wait_bounded(&bars[1], phase1);
            atomicOr(P.err, ERRW_WAIT_TIMEOUT);
        }
        return;
    }
    if (cur_lag >= 0) flush_hist(hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
    add_stats(P.stats, n_cand, n_rech);
}

// ---------------------------------------------------------------------------
// Plain FP64 kernel: the reference arithmetic for every pair
// ---------------------------------------------------------------------------
template <bool TRI>
__global__ void __launch_bounds__(NT, 2) k_pairs_f64(const PairLaunch P)
{
    extern __shared__ __align__(128) unsigned char smem[];
    double *jx = reinterpret_cast<double *>(smem);
    double *jy = jx + TJ64;
    double *jz = jy + TJ64;
    int *jt = reinterpret_cast<int *>(jz + TJ64);
    unsigned *hist = reinterpret_cast<unsigned *>(jt + TJ64);
    unsigned short *chtab = reinterpret_cast<unsigned short *>(hist + P.nch * P.nbin);

    const int tid = threadIdx.x;
    const int hlen = P.nch * P.nbin;
    const int half = P.nch / 2;
    for (int i = tid; i < hlen; i += NT) hist[i] = 0u;
    for (int i = tid; i < P.ntypes * P.ntypes; i += NT) chtab[i] = P.chtab[i];
    __syncthreads();

    const long long per = (P.n_items + gridDim.x - 1) / gridDim.x;
    const long long it0 = (long long)blockIdx.x * per;
    const long long it1 = min(it0 + per, P.n_items);
    const long long N = P.N;
    const long long flush_every = items_per_flush(TI64, P.N);
    int cur_lag = -1;
    long long since_flush = 0;

    for (long long item = it0; item < it1; ++item) {
        int lag_idx, itile, k;
        decompose(item, P, lag_idx, itile, k);
        if (lag_idx != cur_lag || since_flush >= flush_every) {
            if (cur_lag >= 0)
                flush_hist(hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
            cur_lag = lag_idx;
            since_flush = 0;
        }
        ++since_flush;
        const long long fo = P.primo + (long long)k * P.skip;
        const long long fl = fo + (long long)lag_idx * P.every;
        double box[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) box[q] = P.box64[fo * 9 + q];

        double xi[R64], yi[R64], zi[R64];
        int ti[R64], ia[R64];
        bool vi[R64];
#pragma unroll
        for (int r = 0; r < R64; ++r) {
            ia[r] = P.a0 + itile * TI64 + r * NT + tid;
            vi[r] = ia[r] < P.a1;
            int a = vi[r] ? ia[r] : P.a0;
            const double *p = P.pos64 + (fo * N + a) * 3;
            xi[r] = p[0]; yi[r] = p[1]; zi[r] = p[2];
            // type ids travel in the FP32 frame's w lane
            ti[r] = __float_as_int(P.pos32[fo * N + a].w);
        }
        for (int jbase = 0; jbase < P.N; jbase += TJ64) {
            const int tj = min(TJ64, P.N - jbase);
            __syncthreads();
            for (int q = tid; q < tj; q += NT) {
                const double *p = P.pos64 + (fl * N + jbase + q) * 3;
                jx[q] = p[0]; jy[q] = p[1]; jz[q] = p[2];
                jt[q] = __float_as_int(P.pos32[fl * N + jbase + q].w);
            }
            __syncthreads();
            for (int jj = 0; jj < tj; ++jj) {
                const double x = jx[jj], y = jy[jj], z = jz[jj];
                const int tj_ = jt[jj];
#pragma unroll
                for (int r = 0; r < R64; ++r) {
                    if (!vi[r]) continue;
                    double d2 = ref_d2<TRI>(xi[r], yi[r], zi[r], x, y, z, box, P.err);
                    int b = ref_bin(d2, P.rmin, P.dr, P.rmin2, P.rmax2, P.nbin);
                    if (b >= 0) {
                        int ch = chtab[ti[r] * P.ntypes + tj_] + (ia[r] == jbase + jj ? half : 0);
                        atomicAdd(hist + ch * P.nbin + b, 1u);
                    }
                }
            }
        }
    }
    if (cur_lag >= 0) flush_hist(hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
}

// ---------------------------------------------------------------------------
// Frame residency: FP64 min/max per axis and FP64 AoS -> FP32 {x,y,z,type}
// ---------------------------------------------------------------------------
__global__ void k_minmax(const double *__restrict__ pos, size_t natoms_total, double *out,
                         unsigned *nonfinite)
{
    __shared__ double sm[6][NT];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    unsigned bad = 0;
    for (size_t a = blockIdx.x * (size_t)NT + threadIdx.x; a < natoms_total;
         a += (size_t)gridDim.x * NT) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double v = pos[a * 3 + k];
            if (!isfinite(v)) { ++bad; continue; }
            mn[k] = fmin(mn[k], v);
            mx[k] = fmax(mx[k], v);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) { sm[k][threadIdx.x] = mn[k]; sm[3 + k][threadIdx.x] = mx[k]; }
    __syncthreads();
    for (int s = NT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                sm[k][threadIdx.x] = fmin(sm[k][threadIdx.x], sm[k][threadIdx.x + s]);
                sm[3 + k][threadIdx.x] = fmax(sm[3 + k][threadIdx.x], sm[3 + k][threadIdx.x + s]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) out[blockIdx.x * 6 + threadIdx.x] = sm[threadIdx.x][0];
    if (bad) atomicAdd(nonfinite, bad);
}

__global__ void k_convert(const double *__restrict__ pos, const int *__restrict__ types, size_t T,
                          size_t N, double cx, double cy, double cz, float4 *__restrict__ out)
{
    size_t total = T * N;
    for (size_t a = blockIdx.x * (size_t)blockDim.x + threadIdx.x; a < total;
         a += (size_t)gridDim.x * blockDim.x) {
        const double *p = pos + a * 3;
        float4 v;
        v.x = __double2float_rn(__dsub_rn(p[0], cx));
        v.y = __double2float_rn(__dsub_rn(p[1], cy));
        v.z = __double2float_rn(__dsub_rn(p[2], cz));
        v.w = __int_as_float(types[a % N]);
        out[a] = v;
    }
}

__global__ void k_zero_u64(unsigned long long *p, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = 0ull;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static int cuda_ok(cudaError_t e) { return e == cudaSuccess ? 0 : -1; }

int launch_minmax(const double *pos64, size_t natoms_total, double *d_out6, unsigned *d_nonfinite,
                  cudaStream_t s)
{
    // fixed grid so the host knows how many partial results to reduce
    k_minmax<<<256, NT, 0, s>>>(pos64, natoms_total, d_out6, d_nonfinite);
    return cuda_ok(cudaGetLastError());
}

int launch_convert(const double *pos64, const int *types, size_t T, size_t N, double cx,
                   double cy, double cz, float4 *pos32, cudaStream_t s)
{
    size_t total = T * N;
    int blocks = (int)((total + NT - 1) / NT);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    k_convert<<<blocks, NT, 0, s>>>(pos64, types, T, N, cx, cy, cz, pos32);
    return cuda_ok(cudaGetLastError());
}

int launch_zero_u64(unsigned long long *p, size_t n, cudaStream_t s)
{
    if (n == 0) return 0;
    int blocks = (int)((n + NT - 1) / NT);
    if (blocks > 1024) blocks = 1024;
    k_zero_u64<<<blocks, NT, 0, s>>>(p, n);
    return cuda_ok(cudaGetLastError());
}

int pairs_smem_bytes(int kind, int nch, int nbin, int ntypes)
{
    size_t hist = (size_t)nch * nbin * 4, tab = (size_t)ntypes * ntypes * 2;
    size_t b;
    if (kind == 0) b = 2 * TJ32 * sizeof(float4) + 32 + (size_t)nbin * 8 + hist + tab;
    else b = (size_t)TJ64 * (3 * 8 + 4) + hist + tab;
    return (int)((b + 127) / 128 * 128);
}

template <typename K>
static int launch_persistent(K kernel, const PairLaunch &P, int smem, int num_sms, cudaStream_t s)
{
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
        cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, NT, smem) != cudaSuccess)
        return -1;
    if (per_sm < 1) return -2;
    long long grid = (long long)num_sms * per_sm;
    if (grid > P.n_items) grid = P.n_items;
    if (grid < 1) grid = 1;
    kernel<<<(unsigned)grid, NT, smem, s>>>(P);
    return cuda_ok(cudaGetLastError());
}

int launch_pairs(const PairLaunch &P, int kind, bool wrapcheck, int num_sms, cudaStream_t s,
                 size_t *smem_bytes_out)
{
    const int smem = pairs_smem_bytes(kind, P.nch, P.nbin, P.ntypes);
    if (smem_bytes_out) *smem_bytes_out = (size_t)smem;
    if (P.n_items <= 0) return 0;
    if (kind == 0) {
        if (P.tric) {
            return wrapcheck ? launch_persistent(k_pairs_f32<true, true>, P, smem, num_sms, s)
                             : launch_persistent(k_pairs_f32<true, false>, P, smem, num_sms, s);
        }
        return wrapcheck ? launch_persistent(k_pairs_f32<false, true>, P, smem, num_sms, s)
                         : launch_persistent(k_pairs_f32<false, false>, P, smem, num_sms, s);
    }
    return P.tric ? launch_persistent(k_pairs_f64<true>, P, smem, num_sms, s)
                  : launch_persistent(k_pairs_f64<false>, P, smem, num_sms, s);
}

}  // namespace gofr
