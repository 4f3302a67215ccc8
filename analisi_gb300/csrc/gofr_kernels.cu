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
// only when the lag changes (or before a u32 bin could overflow).
//
// FP32 kernel, per item: each thread holds R first atoms (frame `origin`)
// in registers, duplicated into f32x2 pairs; the CTA streams the second atoms
// (frame `origin+lag`, SoA x|y|z blocks plus u8 types) through shared memory
// in tiles of TJ atoms, double buffered with 1-D TMA bulk copies completed on
// mbarriers.  Distances are computed two second-atoms per packed f32x2
// instruction.  The rare pairs that land inside the accept window (plus its
// error bound) are appended to per-thread slots in shared memory and binned
// later by the whole warp, so the hot loop never diverges; pairs whose FP32
// bin cannot be certified go to a per-CTA queue recomputed in FP64 by all
// threads together at the end of the item.
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "gofr_device.cuh"
#include "gofr_internal.h"

namespace gofr {

constexpr int NT = 256;       // threads per CTA
constexpr int R32 = 4;        // first atoms per thread, FP32 kernel
constexpr int TI32 = NT * R32;
constexpr int TJ32 = 1024;    // second atoms per shared-memory tile
constexpr int SLOTS = 16;     // candidate slots per thread
constexpr int QCAP = 1024;    // FP64 recheck queue entries per CTA
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
// Adds one count to bin b of channel ch: the shared-memory histogram, or the
// lag's u64 counts in global memory when the histogram does not fit (ghist).
__device__ __forceinline__ void hist_add(unsigned *hist, unsigned long long *gcounts, int ch,
                                         int nbin, int b)
{
    if (gcounts) atomicAdd(gcounts + ch * nbin + b, 1ull);
    else atomicAdd(hist + ch * nbin + b, 1u);
}

template <bool TRI>
__device__ __forceinline__ void recheck_pair(const double *__restrict__ pos64,
                                             const double *__restrict__ box64, long long N,
                                             long long fo, long long fl, int ia, int ja,
                                             unsigned *hist, int ch, int nbin, double rmin,
                                             double dr, double rmin2, double rmax2,
                                             unsigned *err, unsigned long long *gcounts = nullptr)
{
    const double *xi = pos64 + (fo * N + ia) * 3;
    const double *xj = pos64 + (fl * N + ja) * 3;
    const double *box = box64 + fo * 9;
    double d2 = ref_d2<TRI>(xi[0], xi[1], xi[2], xj[0], xj[1], xj[2], box, err);
    int b = ref_bin(d2, rmin, dr, rmin2, rmax2, nbin);
    if (b >= 0 && GOFR_CHECK(b < nbin && ch >= 0, err)) hist_add(hist, gcounts, ch, nbin, b);
}

// ---------------------------------------------------------------------------
// packed f32x2 arithmetic (PTX ISA add/sub/mul/fma .f32x2, sm_100+)
// ---------------------------------------------------------------------------
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
__device__ __forceinline__ f2 f2add(f2 a, f2 b)
{
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
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

// Box constants of one origin frame, duplicated into both f32x2 lanes.
struct Box2 {
    f2 invL[3], negL[3];
    f2 negT[3];   // -{xy, xz, yz}
};

// Minimum-image d2 of (i, j0) and (i, j1) in one f32x2 lane pair.
// WCHK: also reports, per lane, whether some wrap quotient lay within the
// certified bound of a half-integer (bits 0 and 1 of *wflag).
template <bool TRI, bool WCHK>
__device__ __forceinline__ f2 pair2(f2 xi, f2 yi, f2 zi, f2 xj, f2 yj, f2 zj, const Box2 &b,
                                    float wlim, unsigned *wflag)
{
    const f2 MAG = f2pk(12582912.0f, 12582912.0f);  // 1.5*2^23: rounds to integer
    f2 dx = f2sub(xi, xj), dy = f2sub(yi, yj), dz = f2sub(zi, zj);
    if (TRI) {
        f2 kz;
        if (WCHK) {
            f2 q = f2mul(dz, b.invL[2]);
            kz = f2sub(f2add(q, MAG), MAG);
            float a0, a1;
            f2up(f2sub(q, kz), a0, a1);
            *wflag |= (fabsf(a0) > wlim ? 1u : 0u) | (fabsf(a1) > wlim ? 2u : 0u);
        } else {
            kz = f2sub(f2fma(dz, b.invL[2], MAG), MAG);
        }
        dz = f2fma(kz, b.negL[2], dz);
        dy = f2fma(kz, b.negT[2], dy);
        dx = f2fma(kz, b.negT[1], dx);
        f2 ky;
        if (WCHK) {
            f2 q = f2mul(dy, b.invL[1]);
            ky = f2sub(f2add(q, MAG), MAG);
            float a0, a1;
            f2up(f2sub(q, ky), a0, a1);
            *wflag |= (fabsf(a0) > wlim ? 1u : 0u) | (fabsf(a1) > wlim ? 2u : 0u);
        } else {
            ky = f2sub(f2fma(dy, b.invL[1], MAG), MAG);
        }
        dy = f2fma(ky, b.negL[1], dy);
        dx = f2fma(ky, b.negT[0], dx);
        f2 kx;
        if (WCHK) {
            f2 q = f2mul(dx, b.invL[0]);
            kx = f2sub(f2add(q, MAG), MAG);
            float a0, a1;
            f2up(f2sub(q, kx), a0, a1);
            *wflag |= (fabsf(a0) > wlim ? 1u : 0u) | (fabsf(a1) > wlim ? 2u : 0u);
        } else {
            kx = f2sub(f2fma(dx, b.invL[0], MAG), MAG);
        }
        dx = f2fma(kx, b.negL[0], dx);
    } else {
        f2 kx, ky, kz;
        if (WCHK) {
            f2 qx = f2mul(dx, b.invL[0]), qy = f2mul(dy, b.invL[1]), qz = f2mul(dz, b.invL[2]);
            kx = f2sub(f2add(qx, MAG), MAG);
            ky = f2sub(f2add(qy, MAG), MAG);
            kz = f2sub(f2add(qz, MAG), MAG);
            float a0, a1, c0, c1, e0, e1;
            f2up(f2sub(qx, kx), a0, a1);
            f2up(f2sub(qy, ky), c0, c1);
            f2up(f2sub(qz, kz), e0, e1);
            bool w0 = fabsf(a0) > wlim || fabsf(c0) > wlim || fabsf(e0) > wlim;
            bool w1 = fabsf(a1) > wlim || fabsf(c1) > wlim || fabsf(e1) > wlim;
            *wflag |= (w0 ? 1u : 0u) | (w1 ? 2u : 0u);
        } else {
            kx = f2sub(f2fma(dx, b.invL[0], MAG), MAG);
            ky = f2sub(f2fma(dy, b.invL[1], MAG), MAG);
            kz = f2sub(f2fma(dz, b.invL[2], MAG), MAG);
        }
        dx = f2fma(kx, b.negL[0], dx);
        dy = f2fma(ky, b.negL[1], dy);
        dz = f2fma(kz, b.negL[2], dz);
    }
    f2 d2 = f2mul(dx, dx);
    d2 = f2fma(dy, dy, d2);
    d2 = f2fma(dz, dz, d2);
    return d2;
}

// Shared-memory layout of the FP32 kernel (byte offsets).
struct F32Smem {
    int jx, jt, bars, flag, rqn, win, hist, chtab, slots, rq, total;
    __host__ __device__ F32Smem(int nbin, int nch, int ntypes, bool ghist = false)
    {
        int o = 0;
        jx = o;    o += 2 * 3 * TJ32 * 4;        // [2][3][TJ] floats
        jt = o;    o += 2 * TJ32;                // [2][TJ] u8 types
        bars = o;  o += 16;                      // 2 mbarriers
        flag = o;  o += 8;
        rqn = o;   o += 8;
        slots = o; o += SLOTS * NT * 8;          // [SLOTS][NT] uint2
        rq = o;    o += QCAP * 16;               // [QCAP] uint4
        win = o;   o += nbin * 8;                // [nbin] float2
        hist = o;  o += ghist ? 0 : nch * nbin * 4;  // [nch][nbin] u32
        chtab = o; o += ntypes * ntypes * 2;     // [ntypes][ntypes] u16
        total = (o + 127) / 128 * 128;
    }
};

// ---------------------------------------------------------------------------
// FP32 bulk + FP64 edge recheck
// ---------------------------------------------------------------------------
//
// Per pair (orthorhombic): FP32 difference, per axis an FMA with a 1.5*2^23
// offset and a subtraction that round d/L to the nearest integer k, an FMA
// d - k*L (L rounded to FP32; its rounding is part of the bound), then d2 by
// one multiply and two FMAs -- 15 FP32 operations issued as f32x2 for two
// second atoms at once -- and one compare against hi_f.  The bound behind
// hi_f, lo_f and the per-bin windows is derived on the host (gofr_capi.cu,
// certify()).

// Shared-memory views of the FP32 kernels.
struct F32Views {
    float *jx;
    unsigned char *jt;
    uint64_t *bars;
    int *sflag, *rqn;
    uint2 *slots;
    uint4 *rq;
    float2 *win;
    unsigned *hist;
    unsigned short *chtab;
    __device__ F32Views(unsigned char *smem, const F32Smem &L)
        : jx(reinterpret_cast<float *>(smem + L.jx)), jt(smem + L.jt),
          bars(reinterpret_cast<uint64_t *>(smem + L.bars)),
          sflag(reinterpret_cast<int *>(smem + L.flag)),
          rqn(reinterpret_cast<int *>(smem + L.rqn)),
          slots(reinterpret_cast<uint2 *>(smem + L.slots)),
          rq(reinterpret_cast<uint4 *>(smem + L.rq)),
          win(reinterpret_cast<float2 *>(smem + L.win)),
          hist(reinterpret_cast<unsigned *>(smem + L.hist)),
          chtab(reinterpret_cast<unsigned short *>(smem + L.chtab))
    {
    }
};

// Per-thread state carried across items: mbarrier phases and counters.
struct F32Thread {
    unsigned phase0 = 0u, phase1 = 0u;
    unsigned long long n_cand = 0, n_rech = 0;
};

__device__ __forceinline__ void f32_init_barriers(const F32Views &V)
{
    if (threadIdx.x == 0) {
        mbar_init(&V.bars[0], 1);
        mbar_init(&V.bars[1], 1);
        *V.sflag = 0;
        *V.rqn = 0;
        fence_mbar_init();
    }
}

// A bounded wait ran out: a copy may still be in flight into either buffer
// (the one waited for, and the prefetch of the next tile).  Give both a
// bounded chance to land before the CTA exits and its shared memory is reused.
__device__ __forceinline__ void f32_abort(const F32Views &V, const F32Thread &th, unsigned *err,
                                          unsigned cap = WAIT_CAP)
{
    if (threadIdx.x == 0) {
        mbar_wait_bounded(&V.bars[0], th.phase0, cap);
        mbar_wait_bounded(&V.bars[1], th.phase1, cap);
        atomicOr(err, ERRW_WAIT_TIMEOUT);
    }
}

// Debug builds: the bounded-wait test (P.dbg_stall) issues no copy at all, so
// nothing is ever in flight when its short wait gives up.
#ifdef GOFR_DEBUG_BOUNDS
#define GOFR_STALL(P) ((P).dbg_stall != 0)
#else
#define GOFR_STALL(P) false
#endif

// One item: the first atoms of tile `itile` at origin k against every second
// atom at lag lag_idx, binned into V.hist.  Returns false if a bounded wait
// ran out (the caller aborts the CTA).  All threads of the CTA call it.
template <bool TRI, bool WCHK>
__device__ __forceinline__ bool f32_item(const PairLaunch &P, const F32Views &V, F32Thread &th,
                                         int lag_idx, int itile, int k)
{
    const int tid = threadIdx.x;
    const int half = P.nch / 2;
    const long long N = P.N, NP = P.NP;
    const int nchunks = (P.N + TJ32 - 1) / TJ32;
    const float hi_f = P.hi_f;
    uint2 *const my_slots = V.slots + tid;
    const long long fo = P.primo + (long long)k * P.skip;
    const long long fl = fo + (long long)lag_idx * P.every;
    unsigned long long *const gc =
        P.ghist ? P.counts + (long long)lag_idx * P.every * P.nch * P.nbin : nullptr;
    Box2 bx;
    {
        const Box32 b = P.box32[fo];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            bx.invL[a] = f2pk(b.invL[a], b.invL[a]);
            bx.negL[a] = f2pk(-b.L[a], -b.L[a]);
            bx.negT[a] = f2pk(-b.tilt[a], -b.tilt[a]);
        }
    }
    // first atoms of this item
    const int ia0 = P.a0 + itile * TI32 + tid;
    f2 xi[R32], yi[R32], zi[R32];
    int ti[R32];
    const float *fi = P.pos32 + fo * 3 * NP;
#pragma unroll
    for (int r = 0; r < R32; ++r) {
        const int ia = ia0 + r * NT;
        float x, y, z;
        if (ia < P.a1) {
            x = fi[ia]; y = fi[NP + ia]; z = fi[2 * NP + ia];
            ti[r] = P.types8[ia];
        } else {
            // no atom: NaN never passes d2 <= hi_f nor the wrap check
            x = y = z = __int_as_float(0x7fc00000);
            ti[r] = 0;
        }
        xi[r] = f2pk(x, x); yi[r] = f2pk(y, y); zi[r] = f2pk(z, z);
    }

    const float *fj = P.pos32 + fl * 3 * NP;
    int cnt = 0;
    const bool stall = GOFR_STALL(P);
    const unsigned wait_cap = stall ? DBG_WAIT_CAP : WAIT_CAP;
    __syncthreads();  // previous item done with both buffers
    if (tid == 0 && stall) {
        mbar_arrive_expect_tx(&V.bars[0], 16u);  // bytes no copy will bring
    } else if (tid == 0) {
        const int tj = min(TJ32, P.N);
        const unsigned fb = (unsigned)(((tj + 3) & ~3) * 4), tb = (unsigned)((tj + 15) & ~15);
        mbar_arrive_expect_tx(&V.bars[0], 3 * fb + tb);
        bulk_g2s(V.jx, fj, fb, &V.bars[0]);
        bulk_g2s(V.jx + TJ32, fj + NP, fb, &V.bars[0]);
        bulk_g2s(V.jx + 2 * TJ32, fj + 2 * NP, fb, &V.bars[0]);
        bulk_g2s(V.jt, P.types8, tb, &V.bars[0]);
    }
    for (int c = 0; c < nchunks; ++c) {
        const int b = c & 1;
        const int jbase = c * TJ32;
        if (tid == 0 && c + 1 < nchunks && !stall) {
            const int nb = jbase + TJ32;
            const int tj = min(TJ32, P.N - nb);
            const unsigned fb = (unsigned)(((tj + 3) & ~3) * 4);
            const unsigned tb = (unsigned)((tj + 15) & ~15);
            float *dst = V.jx + (b ^ 1) * 3 * TJ32;
            mbar_arrive_expect_tx(&V.bars[b ^ 1], 3 * fb + tb);
            bulk_g2s(dst, fj + nb, fb, &V.bars[b ^ 1]);
            bulk_g2s(dst + TJ32, fj + NP + nb, fb, &V.bars[b ^ 1]);
            bulk_g2s(dst + 2 * TJ32, fj + 2 * NP + nb, fb, &V.bars[b ^ 1]);
            bulk_g2s(V.jt + (b ^ 1) * TJ32, P.types8 + nb, tb, &V.bars[b ^ 1]);
        }
        const bool ok = mbar_wait_bounded(&V.bars[b], b ? th.phase1 : th.phase0, wait_cap);
        if (ok) { if (b) th.phase1 ^= 1u; else th.phase0 ^= 1u; }
        else atomicOr(V.sflag, 1);
        __syncthreads();
        if (*V.sflag) return false;

        const int tj = min(TJ32, P.N - jbase);
        const float *bxp = V.jx + b * 3 * TJ32;
        const unsigned char *btp = V.jt + b * TJ32;

        // Bins every slot of this warp's lanes (all lanes take part; each
        // processes its own slots, two per round so that their shared-memory
        // load chains overlap), then empties them.  Shared-histogram updates
        // are predicated reductions; the rare FP64 rechecks sit behind one
        // warp-uniform branch.
        auto warp_flush = [&]() {
            const int maxc = __reduce_max_sync(0xffffffffu, (unsigned)cnt);
            for (int q0 = 0; q0 < maxc; q0 += 2) {
                uint2 e[2];
                bool v[2], ok[2], need[2];
                int ch[2], bi[2], ia[2], ja[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    v[u] = q0 + u < cnt;
                    e[u] = v[u] ? my_slots[(q0 + u) * NT] : make_uint2(0x7f800000u, 0u);
                }
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const float d2 = __uint_as_float(e[u].x);
                    const int r = e[u].y & 3;
                    const int jj = (e[u].y >> 2) & 0x1fff;
                    ia[u] = ia0 + r * NT;
                    ja[u] = jbase + jj;
                    int t_i = ti[0];
#pragma unroll
                    for (int rr = 1; rr < R32; ++rr) t_i = (r == rr) ? ti[rr] : t_i;
                    ch[u] = V.chtab[t_i * P.ntypes + btp[jj]] + (ia[u] == ja[u] ? half : 0);
                    const bool wrap = WCHK && (e[u].y >> 31);  // minimum image not certain
                    const int b_ = __float2int_rd(
                        __fmul_rn(__fsub_rn(sqrt_guess(d2), P.rmin_f), P.inv_dr_f));
                    bi[u] = min(max(b_, 0), P.nbin - 1);
                    const float2 w = V.win[bi[u]];
                    const bool test = v[u] && !wrap && d2 >= P.lo_f;
                    const bool inw = d2 >= w.x && d2 <= w.y;
                    ok[u] = test && inw &&
                            GOFR_CHECK(ch[u] >= 0 && ch[u] < P.nch && bi[u] >= 0 &&
                                           bi[u] < P.nbin && jj < tj && ia[u] < P.a1,
                                       P.err);
                    need[u] = (v[u] && wrap) || (test && !inw);
                }
                if (gc) {
#pragma unroll
                    for (int u = 0; u < 2; ++u)
                        if (ok[u]) atomicAdd(gc + ch[u] * P.nbin + bi[u], 1ull);
                } else {
#pragma unroll
                    for (int u = 0; u < 2; ++u)
                        red_shared_add1_if(smem_u32(V.hist + ch[u] * P.nbin + bi[u]), ok[u]);
                }
                if (__any_sync(0xffffffffu, need[0] || need[1])) {
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        if (!need[u]) continue;
                        ++th.n_rech;
                        const int slot = atomicAdd(V.rqn, 1);
                        if (slot < QCAP) {
                            V.rq[slot] =
                                make_uint4((unsigned)ia[u], (unsigned)ja[u], (unsigned)ch[u], 0u);
                        } else {
                            recheck_pair<TRI>(P.pos64, P.box64, N, fo, fl, ia[u], ja[u], V.hist,
                                              ch[u], P.nbin, P.rmin, P.dr, P.rmin2, P.rmax2, P.err,
                                              gc);
                        }
                    }
                }
            }
            th.n_cand += cnt;
            cnt = 0;
        };

        for (int jj = 0; jj < tj; jj += 4) {
            const float4 X = *reinterpret_cast<const float4 *>(bxp + jj);
            const float4 Y = *reinterpret_cast<const float4 *>(bxp + TJ32 + jj);
            const float4 Z = *reinterpret_cast<const float4 *>(bxp + 2 * TJ32 + jj);
            const f2 xa = f2pk(X.x, X.y), xb = f2pk(X.z, X.w);
            const f2 ya = f2pk(Y.x, Y.y), yb = f2pk(Y.z, Y.w);
            const f2 za = f2pk(Z.x, Z.y), zb = f2pk(Z.z, Z.w);
#pragma unroll
            for (int r = 0; r < R32; ++r) {
                unsigned wa = 0u, wb = 0u;
                const f2 da = pair2<TRI, WCHK>(xi[r], yi[r], zi[r], xa, ya, za, bx, P.wlim, &wa);
                const f2 db = pair2<TRI, WCHK>(xi[r], yi[r], zi[r], xb, yb, zb, bx, P.wlim, &wb);
                float d0, d1, d2v, d3;
                f2up(da, d0, d1);
                f2up(db, d2v, d3);
                const unsigned m0 = (unsigned)((jj << 2) | r);
                if (d0 <= hi_f || (WCHK && (wa & 1u))) {
                    my_slots[cnt * NT] = make_uint2(__float_as_uint(d0), m0 | (WCHK && (wa & 1u) ? 0x80000000u : 0u));
                    ++cnt;
                }
                if (d1 <= hi_f || (WCHK && (wa & 2u))) {
                    my_slots[cnt * NT] = make_uint2(__float_as_uint(d1), (m0 + 4u) | (WCHK && (wa & 2u) ? 0x80000000u : 0u));
                    ++cnt;
                }
                if (d2v <= hi_f || (WCHK && (wb & 1u))) {
                    my_slots[cnt * NT] = make_uint2(__float_as_uint(d2v), (m0 + 8u) | (WCHK && (wb & 1u) ? 0x80000000u : 0u));
                    ++cnt;
                }
                if (d3 <= hi_f || (WCHK && (wb & 2u))) {
                    my_slots[cnt * NT] = make_uint2(__float_as_uint(d3), (m0 + 12u) | (WCHK && (wb & 2u) ? 0x80000000u : 0u));
                    ++cnt;
                }
                if (!GOFR_CHECK(cnt <= SLOTS, P.err)) cnt = SLOTS;
                if (__any_sync(0xffffffffu, cnt > SLOTS - 4)) warp_flush();
            }
        }
        if (__any_sync(0xffffffffu, cnt > 0)) warp_flush();
        __syncthreads();  // all reads of buffer b done before it is refilled
        // drain the FP64 recheck queue when half full (uniform decision)
        if (*V.rqn > QCAP / 2) {
            const int n = min(*V.rqn, QCAP);
            for (int q = tid; q < n; q += NT) {
                const uint4 e = V.rq[q];
                recheck_pair<TRI>(P.pos64, P.box64, N, fo, fl, (int)e.x, (int)e.y, V.hist,
                                  (int)e.z, P.nbin, P.rmin, P.dr, P.rmin2, P.rmax2, P.err, gc);
            }
            __syncthreads();
            if (tid == 0) *V.rqn = 0;
            __syncthreads();
        }
    }
    // end of item: the queue refers to this item's frames
    const int n = min(*V.rqn, QCAP);
    for (int q = tid; q < n; q += NT) {
        const uint4 e = V.rq[q];
        recheck_pair<TRI>(P.pos64, P.box64, N, fo, fl, (int)e.x, (int)e.y, V.hist, (int)e.z,
                          P.nbin, P.rmin, P.dr, P.rmin2, P.rmax2, P.err, gc);
    }
    __syncthreads();
    if (tid == 0) *V.rqn = 0;
    return true;
}

// One trajectory: a persistent grid takes contiguous lag-major item ranges.
template <bool TRI, bool WCHK>
__global__ void __launch_bounds__(NT, 2) k_pairs_f32(const PairLaunch P)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const F32Views V(smem, F32Smem(P.nbin, P.nch, P.ntypes, P.ghist != 0));
    const int tid = threadIdx.x;
    const int hlen = P.ghist ? 0 : P.nch * P.nbin;
    for (int i = tid; i < P.nbin; i += NT) V.win[i] = P.win[i];
    for (int i = tid; i < hlen; i += NT) V.hist[i] = 0u;
    for (int i = tid; i < P.ntypes * P.ntypes; i += NT) V.chtab[i] = P.chtab[i];
    f32_init_barriers(V);
    __syncthreads();

    const long long per = (P.n_items + gridDim.x - 1) / gridDim.x;
    const long long it0 = (long long)blockIdx.x * per;
    const long long it1 = min(it0 + per, P.n_items);
    const long long flush_every = items_per_flush(TI32, P.N);
    int cur_lag = -1;
    long long since_flush = 0;
    F32Thread th;
    for (long long item = it0; item < it1; ++item) {
        int lag_idx, itile, k;
        decompose(item, P, lag_idx, itile, k);
        if (lag_idx != cur_lag || since_flush >= flush_every) {
            if (cur_lag >= 0 && hlen)
                flush_hist(V.hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
            cur_lag = lag_idx;
            since_flush = 0;
        }
        ++since_flush;
        if (!f32_item<TRI, WCHK>(P, V, th, lag_idx, itile, k)) {
            f32_abort(V, th, P.err, GOFR_STALL(P) ? DBG_WAIT_CAP : WAIT_CAP);
            return;
        }
    }
    if (cur_lag >= 0 && hlen)
        flush_hist(V.hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
    add_stats(P.stats, th.n_cand, th.n_rech);
}

// Many trajectories in one persistent launch.  Each CTA pulls work
// descriptors (trajectory, lag, first-atom tile, origin range) from a device
// queue (one atomic counter; descriptors sorted by decreasing cost on the
// host), switches the shared tables when the trajectory changes, and flushes
// its histogram into that trajectory's counts at the end of every descriptor.
template <bool TRI>
__global__ void __launch_bounds__(NT, 2) k_pairs_batch(const PairLaunch *__restrict__ trajs,
                                                       const WorkDesc *__restrict__ work,
                                                       int n_work, unsigned *head, int max_nbin,
                                                       int max_nch, int max_ntypes, unsigned *err,
                                                       unsigned long long *stats)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_next;
    // the current trajectory's parameters live in shared memory: a register
    // copy of the whole struct would crowd out the hot loop
    __shared__ __align__(16) PairLaunch sP;
    const F32Views V(smem, F32Smem(max_nbin, max_nch, max_ntypes));
    const int tid = threadIdx.x;
    for (int i = tid; i < max_nch * max_nbin; i += NT) V.hist[i] = 0u;
    f32_init_barriers(V);
    __syncthreads();
    const PairLaunch &P = sP;
    int cur = -1;
    F32Thread th;
    for (;;) {
        if (tid == 0) s_next = (int)atomicAdd(head, 1u);
        __syncthreads();
        const int idx = s_next;
        __syncthreads();
        if (idx >= n_work) break;
        const WorkDesc w = work[idx];
        if (w.traj != cur) {
            constexpr int words = (int)(sizeof(PairLaunch) / 4);
            const unsigned *src = reinterpret_cast<const unsigned *>(trajs + w.traj);
            for (int i = tid; i < words; i += NT) reinterpret_cast<unsigned *>(&sP)[i] = src[i];
            __syncthreads();
            for (int i = tid; i < P.nbin; i += NT) V.win[i] = P.win[i];
            for (int i = tid; i < P.ntypes * P.ntypes; i += NT) V.chtab[i] = P.chtab[i];
            cur = w.traj;
            __syncthreads();
        }
        const bool wchk = P.wchk != 0;
        for (int k = w.k0; k < w.k1; ++k) {
            const bool ok = wchk ? f32_item<TRI, true>(P, V, th, w.lag_idx, w.itile, k)
                                 : f32_item<TRI, false>(P, V, th, w.lag_idx, w.itile, k);
            if (!ok) {
                f32_abort(V, th, err);
                return;
            }
        }
        const int hlen = P.nch * P.nbin;
        flush_hist(V.hist, hlen, P.counts + (long long)w.lag_idx * P.every * hlen);
    }
    add_stats(stats, th.n_cand, th.n_rech);
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
    const int hlen = P.ghist ? 0 : P.nch * P.nbin;
    unsigned short *chtab = reinterpret_cast<unsigned short *>(hist + hlen);

    const int tid = threadIdx.x;
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
            if (cur_lag >= 0 && hlen)
                flush_hist(hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
            cur_lag = lag_idx;
            since_flush = 0;
        }
        ++since_flush;
        const long long fo = P.primo + (long long)k * P.skip;
        const long long fl = fo + (long long)lag_idx * P.every;
        unsigned long long *const gc =
            P.ghist ? P.counts + (long long)lag_idx * P.every * P.nch * P.nbin : nullptr;
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
            ti[r] = P.types8[a];
        }
        for (int jbase = 0; jbase < P.N; jbase += TJ64) {
            const int tj = min(TJ64, P.N - jbase);
            __syncthreads();
            for (int q = tid; q < tj; q += NT) {
                const double *p = P.pos64 + (fl * N + jbase + q) * 3;
                jx[q] = p[0]; jy[q] = p[1]; jz[q] = p[2];
                jt[q] = P.types8[jbase + q];
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
                        if (GOFR_CHECK(ch >= 0 && ch < P.nch && b < P.nbin, P.err))
                            hist_add(hist, gc, ch, P.nbin, b);
                    }
                }
            }
        }
    }
    if (cur_lag >= 0 && hlen)
        flush_hist(hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
}

// ---------------------------------------------------------------------------
// Frame residency: FP64 min/max per axis and FP64 AoS -> FP32 SoA
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

// [T][N][3] FP64 -> [T][3][NP] FP32 (x-cx | y-cy | z-cz), padding NaN; types -> u8.
__global__ void k_convert(const double *__restrict__ pos, const int *__restrict__ types, size_t T,
                          size_t N, size_t NP, double cx, double cy, double cz,
                          float *__restrict__ out, unsigned char *__restrict__ types8)
{
    const size_t total = T * NP;
    const float qnan = __int_as_float(0x7fc00000);
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total;
         g += (size_t)gridDim.x * blockDim.x) {
        const size_t f = g / NP, a = g - f * NP;
        float x = qnan, y = qnan, z = qnan;
        if (a < N) {
            const double *p = pos + (f * N + a) * 3;
            x = __double2float_rn(__dsub_rn(p[0], cx));
            y = __double2float_rn(__dsub_rn(p[1], cy));
            z = __double2float_rn(__dsub_rn(p[2], cz));
        }
        float *o = out + f * 3 * NP;
        o[a] = x;
        o[NP + a] = y;
        o[2 * NP + a] = z;
        if (f == 0) types8[a] = (unsigned char)(a < N ? types[a] : 0);
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
                   double cy, double cz, float *pos32, unsigned char *types8, cudaStream_t s)
{
    const size_t NP = padded_natoms(N);
    size_t total = T * NP;
    int blocks = (int)((total + NT - 1) / NT);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    k_convert<<<blocks, NT, 0, s>>>(pos64, types, T, N, NP, cx, cy, cz, pos32, types8);
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

int pairs_smem_bytes(int kind, int nch, int nbin, int ntypes, bool ghist)
{
    if (kind == 0) return F32Smem(nbin, nch, ntypes, ghist).total;
    size_t b = (size_t)TJ64 * (3 * 8 + 4) + (ghist ? 0 : (size_t)nch * nbin * 4) +
               (size_t)ntypes * ntypes * 2;
    return (int)((b + 127) / 128 * 128);
}

int pairs_tile_atoms(int kind) { return kind == 0 ? TI32 : TI64; }

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

int batch_smem_bytes(int max_nbin, int max_nch, int max_ntypes)
{
    return F32Smem(max_nbin, max_nch, max_ntypes).total;
}

int prepare_batch(int max_nbin, int max_nch, int max_ntypes, bool tric, int num_sms, int n_work,
                  int *grid_out)
{
    const int smem = batch_smem_bytes(max_nbin, max_nch, max_ntypes);
    auto kernel = tric ? k_pairs_batch<true> : k_pairs_batch<false>;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
        cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, NT, smem) != cudaSuccess)
        return -1;
    if (per_sm < 1) return -2;
    long long grid = (long long)num_sms * per_sm;
    if (grid > n_work) grid = n_work;
    *grid_out = (int)(grid < 1 ? 1 : grid);
    return 0;
}

int launch_batch_grid(const PairLaunch *d_trajs, const WorkDesc *d_work, int n_work,
                      unsigned *d_head, int max_nbin, int max_nch, int max_ntypes, bool tric,
                      unsigned *d_err, unsigned long long *d_stats, int grid, cudaStream_t s)
{
    if (n_work <= 0) return 0;
    const int smem = batch_smem_bytes(max_nbin, max_nch, max_ntypes);
    auto kernel = tric ? k_pairs_batch<true> : k_pairs_batch<false>;
    kernel<<<(unsigned)grid, NT, smem, s>>>(d_trajs, d_work, n_work, d_head, max_nbin, max_nch,
                                            max_ntypes, d_err, d_stats);
    return cuda_ok(cudaGetLastError());
}

int launch_pairs(const PairLaunch &P, int kind, bool wrapcheck, int num_sms, cudaStream_t s,
                 size_t *smem_bytes_out)
{
    const int smem = pairs_smem_bytes(kind, P.nch, P.nbin, P.ntypes, P.ghist != 0);
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
