// Mean square displacement on the resident FP64 frames (the reference's
// MSD<T>::calc_single_th, lib/src/msd.cpp:70-118).
//
// The reference loops lag -> origin -> atom and keeps, per (lag, type), a
// running mean of |x_i(o) - x_i(o+t)|^2 (optionally minus the type's
// centre-of-mass displacement), and of the centres' own squared displacement.
// Here every (origin, lag) item is one CTA: it forms each atom's displacement
// with the reference's FP64 operations, adds its squared components into the
// type's sum with FMAs (atoms visited in type-sorted order, one block
// reduction per type) and writes one partial sum per (lag, origin, type).  A second kernel adds the origins of each
// (lag, type) in a fixed order and divides by the count.  Items are ordered
// origin-major so that consecutive CTAs share the origin frame and slide the
// lagged frame, which keeps the frames they read in L2.
#include <cstdint>
#include <cuda_runtime.h>

#include "gofr_internal.h"

namespace gofr {
namespace msd {

constexpr int NT = 256;

__device__ __forceinline__ double sq3(double dx, double dy, double dz)
{
    // pow(dx,2) + pow(dy,2) + pow(dz,2), left to right (lib/src/msd.cpp:98-100)
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ double block_sum(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < NT / 32; ++k) s = __dadd_rn(s, red[k]);
    __syncthreads();
    return s;  // valid in thread 0
}

__global__ void __launch_bounds__(NT) k_msd_partial(const MsdLaunch M)
{
    __shared__ double red[NT / 32];
    const int fk = M.cm_msd ? 2 * M.ntypes : M.ntypes;
    const long long n_items = (long long)M.n_orig * M.leff;
    for (long long item = blockIdx.x; item < n_items; item += gridDim.x) {
        const int o = (int)(item / M.leff);
        const int lag = (int)(item - (long long)o * M.leff);
        const long long fo = (long long)M.primo + (long long)o * M.skip;
        const long long fl = fo + lag;
        const double *po = M.pos64 + (size_t)fo * M.N * 3;
        const double *pl = M.pos64 + (size_t)fl * M.N * 3;
        double *out = M.partial + ((size_t)lag * M.n_orig + o) * fk;
        for (int k = 0; k < M.ntypes; ++k) {
            double cx = 0.0, cy = 0.0, cz = 0.0;
            if (M.cm_self) {
                const double *co = M.cm + ((size_t)fo * M.ntypes + k) * 3;
                const double *cl = M.cm + ((size_t)fl * M.ntypes + k) * 3;
                cx = __dsub_rn(co[0], cl[0]);
                cy = __dsub_rn(co[1], cl[1]);
                cz = __dsub_rn(co[2], cl[2]);
            }
            double acc = 0.0;
            for (int q = M.tbegin[k] + threadIdx.x; q < M.tbegin[k + 1]; q += NT) {
                const size_t a = (size_t)M.perm[q] * 3;
                double dx = __dsub_rn(po[a], pl[a]);
                double dy = __dsub_rn(po[a + 1], pl[a + 1]);
                double dz = __dsub_rn(po[a + 2], pl[a + 2]);
                if (M.cm_self) {
                    dx = __dsub_rn(dx, cx);
                    dy = __dsub_rn(dy, cy);
                    dz = __dsub_rn(dz, cz);
                }
                // the squares go straight into the sum (three FMAs instead of
                // three products, two additions and one accumulation: the
                // kernel is bound by the FP64 pipe)
                acc = __fma_rn(dz, dz, __fma_rn(dy, dy, __fma_rn(dx, dx, acc)));
            }
            const double s = block_sum(acc, red);
            if (threadIdx.x == 0) out[k] = s;
        }
        if (M.cm_msd && threadIdx.x < M.ntypes) {
            const int k = threadIdx.x;
            const double *co = M.cm + ((size_t)fo * M.ntypes + k) * 3;
            const double *cl = M.cm + ((size_t)fl * M.ntypes + k) * 3;
            out[M.ntypes + k] =
                sq3(__dsub_rn(co[0], cl[0]), __dsub_rn(co[1], cl[1]), __dsub_rn(co[2], cl[2]));
        }
    }
}

// out[lag][c][k] = sum over origins (in order) / count
__global__ void k_msd_final(const MsdLaunch M, double *out)
{
    const int fk = M.cm_msd ? 2 * M.ntypes : M.ntypes;
    const long long n = (long long)M.leff * fk;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        const int lag = (int)(g / fk), c = (int)(g - (long long)lag * fk);
        const double *p = M.partial + (size_t)lag * M.n_orig * fk + c;
        double s = 0.0;
        for (int o = 0; o < M.n_orig; ++o) s = __dadd_rn(s, p[(size_t)o * fk]);
        const double count = c < M.ntypes
                                 ? (double)M.n_orig * (double)(M.tbegin[c + 1] - M.tbegin[c])
                                 : (double)M.n_orig;
        out[g] = __ddiv_rn(s, count);
    }
}

}  // namespace msd

int launch_msd(const MsdLaunch &M, double *out_device, int num_sms, cudaStream_t s)
{
    using namespace msd;
    const long long n_items = (long long)M.n_orig * M.leff;
    if (n_items <= 0) return 0;
    long long grid = n_items;
    if (grid > (long long)num_sms * 64) grid = (long long)num_sms * 64;
    k_msd_partial<<<(unsigned)grid, NT, 0, s>>>(M);
    const long long nout = (long long)M.leff * (M.cm_msd ? 2 : 1) * M.ntypes;
    long long g2 = (nout + NT - 1) / NT;
    if (g2 > (long long)num_sms * 8) g2 = (long long)num_sms * 8;
    k_msd_final<<<(unsigned)g2, NT, 0, s>>>(M, out_device);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gofr
