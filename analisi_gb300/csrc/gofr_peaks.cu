// Peak microbenchmarks for the roofline of the pair kernels.
//
// The FP32 pair kernel is bounded by the FP32 issue rate (one lane operation
// per FADD/FMUL/FFMA, the unit in which its 16 (orthorhombic) or 19
// (triclinic) operations per pair are counted) and, on the in-range
// fraction, by shared-memory atomics.  Neither peak is in the driver's
// measured peaks file, so they are measured here on the device in use.
#include <cstdint>
#include <cuda_runtime.h>

#include "gofr_gb300.h"

namespace gofr {

constexpr int PK_NT = 256;
constexpr int PK_CHAINS = 8;

// Independent FFMA chains: PK_CHAINS accumulators per thread, iters rounds.
__global__ void __launch_bounds__(PK_NT) k_peak_ffma(float *sink, int iters, float a, float b)
{
    float acc[PK_CHAINS];
#pragma unroll
    for (int c = 0; c < PK_CHAINS; ++c) acc[c] = threadIdx.x * 1e-3f + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < PK_CHAINS; ++c) acc[c] = __fmaf_rn(acc[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < PK_CHAINS; ++c) s += acc[c];
    if (s == 1234.5678f) sink[blockIdx.x] = s;  // keeps the chains alive
}

// Shared-memory u32 atomics, each lane on its own bank-distinct word.
__global__ void __launch_bounds__(PK_NT) k_peak_satom(unsigned *sink, int iters)
{
    __shared__ unsigned h[PK_NT * 4];
    for (int i = threadIdx.x; i < PK_NT * 4; i += PK_NT) h[i] = 0;
    __syncthreads();
    unsigned *p = h + threadIdx.x;
    for (int i = 0; i < iters; ++i) {
        atomicAdd(p, 1u);
        atomicAdd(p + PK_NT, 1u);
        atomicAdd(p + 2 * PK_NT, 1u);
        atomicAdd(p + 3 * PK_NT, 1u);
    }
    __syncthreads();
    if (h[threadIdx.x] == 0xdeadbeefu) sink[blockIdx.x] = h[threadIdx.x];
}

}  // namespace gofr

extern "C" int gofr_measure_peaks(int device, double *fp32_lane_ops_per_s,
                                  double *smem_atomics_per_s)
{
    using namespace gofr;
    int prev = -1;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return GOFR_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float *sink = nullptr;
    cudaEvent_t e0, e1;
    int rc = GOFR_OK;
    if (cudaMalloc(&sink, 65536 * sizeof(float)) != cudaSuccess) rc = GOFR_ERR_NOMEM;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    if (rc == GOFR_OK) {
        const int blocks = sms * 8, iters = 1 << 15;
        k_peak_ffma<<<blocks, PK_NT>>>(sink, 64, 1.0001f, 0.5f);  // warm-up
        double best = 0.0;
        for (int rep = 0; rep < 5; ++rep) {
            cudaEventRecord(e0);
            k_peak_ffma<<<blocks, PK_NT>>>(sink, iters, 0.99999f, 1e-3f);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            double ops = (double)blocks * PK_NT * iters * PK_CHAINS;
            if (ms > 0) best = ops / (ms * 1e-3) > best ? ops / (ms * 1e-3) : best;
        }
        if (fp32_lane_ops_per_s) *fp32_lane_ops_per_s = best;
        const int aiters = 1 << 13;
        k_peak_satom<<<blocks, PK_NT>>>(reinterpret_cast<unsigned *>(sink), 16);
        best = 0.0;
        for (int rep = 0; rep < 5; ++rep) {
            cudaEventRecord(e0);
            k_peak_satom<<<blocks, PK_NT>>>(reinterpret_cast<unsigned *>(sink), aiters);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            double ops = (double)blocks * PK_NT * aiters * 4;
            if (ms > 0) best = ops / (ms * 1e-3) > best ? ops / (ms * 1e-3) : best;
        }
        if (smem_atomics_per_s) *smem_atomics_per_s = best;
        if (cudaGetLastError() != cudaSuccess) rc = GOFR_ERR_CUDA;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (prev >= 0) cudaSetDevice(prev);
    return rc;
}
