// Device helpers for the Gofrt kernels: inline-PTX TMA bulk copies and
// mbarriers (sm_90+ forms, compiled for sm_103a), bounded waits, and the FP64
// restatement of the reference's pair arithmetic used by the plain FP64 kernel
// and by the edge recheck of the FP32 kernel.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "gofr_internal.h"

namespace gofr {

// ---------------------------------------------------------------------------
// mbarrier + cp.async.bulk (1-D TMA) wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

// Makes barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// Global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Iteration cap of every spin wait: each try_wait suspends for a bounded,
// hardware-defined time, so the whole wait is bounded (well under a minute).
constexpr unsigned WAIT_CAP = 1u << 20;
// Cap of the waits of the debug builds' bounded-wait test (a barrier that no
// copy completes): the wait and the abort that follows end within microseconds.
constexpr unsigned DBG_WAIT_CAP = 256u;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity,
                                                  unsigned cap = WAIT_CAP)
{
    for (unsigned it = 0; it < cap; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Square root for the bin guess of a candidate only.  The certified window
// test that follows decides whether the pair is counted in the guessed bin,
// so the hardware approximation (a few ulp) is enough: a guess that is wrong
// near a bin edge fails the window test and the pair goes to the FP64
// recheck, exactly as a pair inside a window margin does.
__device__ __forceinline__ float sqrt_guess(float x)
{
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Adds 1 to the shared-memory word at addr when p holds, as one predicated
// reduction: the histogram updates of a warp flush issue without a branch
// (and its convergence bookkeeping) around each of them.
__device__ __forceinline__ void red_shared_add1_if(unsigned addr, bool p)
{
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %1, 0;\n\t@q red.shared.add.u32 [%0], 1;\n\t}"
                 ::"r"(addr), "r"((unsigned)p)
                 : "memory");
}

// ---------------------------------------------------------------------------
// FP64 restatement of the reference pair arithmetic.
// Every operation is an explicitly rounded IEEE intrinsic, so nvcc cannot
// contract a multiply and an add into an FMA: the result is bit-identical to
// the reference compiled without FMA contraction.
// ---------------------------------------------------------------------------

// Cap on the iterations of one axis of the iterative minimum image.  The
// reference loops until |d| <= l/2 (lib/include/basetrajectory.h:236-267);
// finite coordinates need at most |d|/l+1 iterations, and non-finite ones are
// rejected when frames are uploaded, so the cap only guards the GPU.
constexpr int WRAP_CAP = 1 << 20;

// Iterative minimum image, z then y then x, strict '>' (basetrajectory.h:224-268).
template <bool TRI>
__device__ __forceinline__ void ref_min_image(double &d0, double &d1, double &d2, const double *box,
                                              unsigned *err)
{
    const double lh0 = box[3], lh1 = box[4], lh2 = box[5];
    const double L0 = __dmul_rn(lh0, 2.0), L1 = __dmul_rn(lh1, 2.0), L2 = __dmul_rn(lh2, 2.0);
    double xy = 0.0, xz = 0.0, yz = 0.0;
    if (TRI) { xy = box[6]; xz = box[7]; yz = box[8]; }
    int g = 0;
    while (fabs(d2) > lh2) {
        if (d2 < 0.0) {
            d2 = __dadd_rn(d2, L2);
            if (TRI) { d1 = __dadd_rn(d1, yz); d0 = __dadd_rn(d0, xz); }
        } else {
            d2 = __dsub_rn(d2, L2);
            if (TRI) { d1 = __dsub_rn(d1, yz); d0 = __dsub_rn(d0, xz); }
        }
        if (++g > WRAP_CAP) { atomicOr(err, ERRW_WRAP_LOOP); break; }
    }
    g = 0;
    while (fabs(d1) > lh1) {
        if (d1 < 0.0) {
            d1 = __dadd_rn(d1, L1);
            if (TRI) d0 = __dadd_rn(d0, xy);
        } else {
            d1 = __dsub_rn(d1, L1);
            if (TRI) d0 = __dsub_rn(d0, xy);
        }
        if (++g > WRAP_CAP) { atomicOr(err, ERRW_WRAP_LOOP); break; }
    }
    g = 0;
    while (fabs(d0) > lh0) {
        if (d0 < 0.0) d0 = __dadd_rn(d0, L0);
        else d0 = __dsub_rn(d0, L0);
        if (++g > WRAP_CAP) { atomicOr(err, ERRW_WRAP_LOOP); break; }
    }
}

// d2 of the reference (basetrajectory.h:200-219): ((0 + x*x) + y*y) + z*z.
template <bool TRI>
__device__ __forceinline__ double ref_d2(double xi0, double xi1, double xi2, double xj0, double xj1,
                                         double xj2, const double *box, unsigned *err)
{
    double d0 = __dsub_rn(xi0, xj0), d1 = __dsub_rn(xi1, xj1), d2 = __dsub_rn(xi2, xj2);
    ref_min_image<TRI>(d0, d1, d2, box, err);
    double s = __dmul_rn(d0, d0);
    s = __dadd_rn(s, __dmul_rn(d1, d1));
    s = __dadd_rn(s, __dmul_rn(d2, d2));
    return s;
}

// Bin of the reference (lib/src/gofrt.cpp:104,114-118): filter on d2, then
// (int)floorf((float)((sqrt(d2)-rmin)/dr)), kept when 0 <= idx < nbin.
// A NaN quotient is dropped, as an x86-64 build of the reference does
// (cvttss2si yields INT_MIN); CUDA's float->int of NaN would give 0.
__device__ __forceinline__ int ref_bin(double d2, double rmin, double dr, double rmin2,
                                       double rmax2, int nbin)
{
    if (d2 > rmax2 || d2 < rmin2) return -1;
    double d = __dsqrt_rn(d2);
    double q = __ddiv_rn(__dsub_rn(d, rmin), dr);
    float qf = __double2float_rn(q);
    float fl = floorf(qf);
    if (!(fl >= 0.0f) || fl >= 2147483648.0f) return -1;  // negative, NaN, or beyond int
    int idx = (int)fl;
    return ((unsigned)idx < (unsigned)nbin) ? idx : -1;
}

// Lattice translate of p into the axis-aligned cell [lo, lo + L) of an
// upper-triangular box (cell vectors a = (Lx, 0, 0), b = (xy, Ly, 0),
// c = (xz, yz, Lz); tilt = {xy, xz, yz}), in FP64: the z count from one
// quotient and floor, the z, y and x components moved by FMAs, then y, then
// x.  Each FMA rounds once, so w differs from p - (nz c + ny b + nx a) by at
// most 2^-53 (|y1| + |w_y|) in y and 2^-53 (|x1| + |x2| + |w_x|) in x.  A
// quotient that rounds across an integer leaves w just outside the cell.
__device__ __forceinline__ void wrap_tric64(const double p[3], const double lo[3],
                                            const double L[3], const double tilt[3], double w[3])
{
    const double nz = floor(__ddiv_rn(__dsub_rn(p[2], lo[2]), L[2]));
    w[2] = __fma_rn(-nz, L[2], p[2]);
    const double y1 = __fma_rn(-nz, tilt[2], p[1]);
    const double x1 = __fma_rn(-nz, tilt[1], p[0]);
    const double ny = floor(__ddiv_rn(__dsub_rn(y1, lo[1]), L[1]));
    w[1] = __fma_rn(-ny, L[1], y1);
    const double x2 = __fma_rn(-ny, tilt[0], x1);
    const double nx = floor(__ddiv_rn(__dsub_rn(x2, lo[0]), L[0]));
    w[0] = __fma_rn(-nx, L[0], x2);
}

}  // namespace gofr
