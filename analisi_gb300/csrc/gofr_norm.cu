// FP64 normalisation of g(r,t) counts on the device.
//
// From the exact counts of one or several calculate(primo) windows (per
// reference thread partition) to the reference's double result, on the GPU:
//   mode 0  the Gofrt buffer (lib/src/gofrt.cpp:118,127-132): each
//           partition's bin is incr added count times in sequence, the
//           partitions folded in order -- bit for bit the reference's doubles;
//   mode 1  that buffer divided by the shell volume 4 pi / 3 (r+^3 - r-^3),
//           r- = b dr + r0, r+ = (b + 1) dr + r0 (pyanalisi/analysis.py:101-105,
//           hist2gofr);
//   mode 2  mode 1 further divided by the channel's pair density: distinct
//           pairs of types a != b: 2 N_a N_b / V, of one type: N_a (N_a - 1) / V;
//           the self channel of type a: N_a (the self part of the van Hove
//           function as a probability density).
// Every operation is an explicitly rounded FP64 intrinsic (no contraction).
// The cubes are computed in double-double arithmetic and rounded once, so
// each is the correctly rounded cube; numpy's `r ** 3` is within one unit in
// the last place of it, which bounds the difference of modes 1 and 2 from a
// host evaluation (the host states that bound with each result).
#include <cuda_runtime.h>

#include "gofr_internal.h"

namespace gofr {
namespace norm {

// The reference's sum of `k` additions of incr starting from 0, in
// O(binades) steps: within one binade, where s + incr rounds by the same
// exact step delta each time, j additions are one multiply-add (the host
// routine of gofr_capi.cu, repeated_sum, in device intrinsics).
__device__ double repeated_sum(unsigned long long k, double incr)
{
    double s = 0.0;
    while (k > 0) {
        const double n1 = __dadd_rn(s, incr);
        if (n1 == s) return s;  // the sum no longer moves
        if (s == 0.0 || !isfinite(n1)) { s = n1; --k; continue; }
        int e;
        frexp(s, &e);                               // s in [2^(e-1), 2^e)
        const double top = ldexp(1.0, e);           // upper end of the binade
        const double u = ldexp(1.0, e - 53);        // ulp in the binade
        const double r = __ddiv_rn(incr, u);        // exact (power-of-two scaling)
        const double fr = __dsub_rn(r, floor(r));
        if (fr == 0.5 || !(__dsub_rn(top, s) > incr)) { s = n1; --k; continue; }
        const double delta = __dsub_rn(n1, s);      // exact: same binade
        const double jm =
            __dsub_rn(floor(__ddiv_rn(__dsub_rn(__dsub_rn(top, s), incr), delta)), 2.0);
        if (jm < 1.0) { s = n1; --k; continue; }
        const unsigned long long j =
            jm >= __ull2double_rn(k) ? k : (unsigned long long)jm;
        s = __dadd_rn(s, __dmul_rn(__ull2double_rn(j), delta));
        k -= j;
    }
    return s;
}

// Correctly rounded x^3: x^2 = h + l exactly (FMA), x^3 = h x + l x with the
// product h x split exactly again; one final rounding of the sum.
__device__ __forceinline__ double cube_rn(double x)
{
    const double h = __dmul_rn(x, x);
    const double l = __fma_rn(x, x, -h);
    const double p = __dmul_rn(h, x);
    const double e = __fma_rn(h, x, -p);
    return __dadd_rn(p, __dadd_rn(e, __dmul_rn(l, x)));
}

__global__ void k_counts_to_gofr(const NormLaunch L)
{
    const size_t total = (size_t)L.nwin * L.n;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total;
         g += (size_t)gridDim.x * blockDim.x) {
        const size_t w = g / L.n, i = g - w * L.n;
        const unsigned long long *c = L.counts + w * L.n * L.nparts + i;
        double acc = repeated_sum(c[0], L.incr);
        for (int q = 1; q < L.nparts; ++q)
            acc = __dadd_rn(acc, repeated_sum(c[(size_t)q * L.n], L.incr));
        if (L.mode >= 1) {
            const int b = (int)(i % L.nbin);
            const int ch = (int)((i / L.nbin) % L.nch);
            const double rm = __dadd_rn(__dmul_rn((double)b, L.dr), L.r0);
            const double rp = __dadd_rn(__dmul_rn((double)(b + 1), L.dr), L.r0);
            const double vol = __dmul_rn(L.c43pi, __dsub_rn(cube_rn(rp), cube_rn(rm)));
            acc = __ddiv_rn(acc, vol);
            if (L.mode == 2) acc = __ddiv_rn(acc, L.chfac[ch]);
        }
        L.out[g] = acc;
    }
}

}  // namespace norm

int launch_counts_to_gofr(const NormLaunch &L, int num_sms, cudaStream_t s)
{
    const size_t total = (size_t)L.nwin * L.n;
    if (total == 0) return 0;
    size_t blocks = (total + 255) / 256;
    if (blocks > (size_t)num_sms * 8) blocks = (size_t)num_sms * 8;
    norm::k_counts_to_gofr<<<(unsigned)blocks, 256, 0, s>>>(L);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gofr
