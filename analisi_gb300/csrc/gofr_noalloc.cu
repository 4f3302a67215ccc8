// gofr_run_f64_noalloc: the plain FP64 pair kernel for callers that cannot
// allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not available or not
// allowed -- inside a host framework that owns every device byte through its
// own pool, inside a real-time loop that must not allocate, or a plug-in
// whose host has already laid out all device memory.  Such a caller already
// holds its frames, types and result buffer in device memory and only needs
// the computation.
//
// The regular entry points (gofr_set_frames / gofr_run) allocate: they keep
// device copies of the frames and per-run tables.  This entry point instead
// reads the caller's device buffers directly and keeps its only scratch --
// the type-pair channel table and the device error word -- in the
// file-scope array g_noalloc_scratch below (SCRATCH_BYTES = 768 bytes; every
// GPU that loads this library holds it until the process exits).  The
// histogram itself lives in shared memory and is added straight into the
// caller's output.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "gofr_gb300.h"
#include "gofr_device.cuh"

namespace gofr {
namespace noalloc {

constexpr int NT = 256;
constexpr int R = 2;          // first atoms per thread
constexpr int TI = NT * R;
constexpr int TJ = 512;       // second atoms per shared-memory tile
constexpr int MAX_TYPES = 16; // limit set by the channel table's slot below
constexpr int OFF_ERR = 0;    // unsigned error word
constexpr int OFF_CHTAB = 256;  // unsigned short [MAX_TYPES][MAX_TYPES]
constexpr int SCRATCH_BYTES = OFF_CHTAB + MAX_TYPES * MAX_TYPES * 2;
constexpr int MAX_DEVICES = 64;
// bit of the error word: a caller's type id outside 0..ntypes-1
constexpr unsigned ERR_TYPE_ID = 0x100u;

}  // namespace noalloc
}  // namespace gofr

// The scratch of every call on a device.  Host code must not use this name as
// an address: it resolves the device address with cudaGetSymbolAddress once
// per device (scratch_on_current_device) and passes that pointer to the kernel.
static __device__ __align__(256) unsigned char g_noalloc_scratch[gofr::noalloc::SCRATCH_BYTES];

namespace gofr {
namespace noalloc {

struct Launch {
    const double *pos;             // [T][N][3] caller's device frames
    const double *box;             // [T][box_stride] caller's device boxes, internal format
    int box_stride;                // 6 or 9
    const int *types;              // [N] caller's device type ids
    unsigned long long *counts;    // [leff][nch][nbin] caller's device output
    unsigned char *scratch;        // device address of g_noalloc_scratch
    int N, nbin, nch, ntypes;
    int n_lags, every, n_orig, skip;
    long long primo;
    int n_itiles;
    long long n_items;
    double rmin, dr, rmin2, rmax2;
};

__device__ __forceinline__ void flush(unsigned *hist, int len, unsigned long long *gout)
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

// Same arithmetic as the plain FP64 pair kernel (reference semantics for every
// pair, lib/src/gofrt.cpp:96-122), reading the caller's buffers directly.
template <bool TRI>
__global__ void __launch_bounds__(NT, 2) k_pairs_f64_noalloc(const Launch P)
{
    extern __shared__ __align__(128) unsigned char smem[];
    double *jx = reinterpret_cast<double *>(smem);
    double *jy = jx + TJ;
    double *jz = jy + TJ;
    int *jt = reinterpret_cast<int *>(jz + TJ);
    unsigned *hist = reinterpret_cast<unsigned *>(jt + TJ);
    unsigned short *chtab = reinterpret_cast<unsigned short *>(hist + P.nch * P.nbin);
    unsigned *err = reinterpret_cast<unsigned *>(P.scratch + OFF_ERR);
    const unsigned short *gtab = reinterpret_cast<const unsigned short *>(P.scratch + OFF_CHTAB);

    const int tid = threadIdx.x;
    const int hlen = P.nch * P.nbin;
    const int half = P.nch / 2;
    for (int i = tid; i < hlen; i += NT) hist[i] = 0u;
    for (int i = tid; i < P.ntypes * P.ntypes; i += NT) chtab[i] = gtab[i];
    __syncthreads();

    const long long per = (P.n_items + gridDim.x - 1) / gridDim.x;
    const long long it0 = (long long)blockIdx.x * per;
    const long long it1 = min(it0 + per, P.n_items);
    const long long N = P.N;
    // no u32 shared bin may overflow: one item adds at most TI*N hits to a bin
    long long flush_every = (1ll << 31) / ((long long)TI * (N > 0 ? N : 1));
    if (flush_every < 1) flush_every = 1;
    int cur_lag = -1;
    long long since = 0;
    for (long long item = it0; item < it1; ++item) {
        const long long per_lag = (long long)P.n_itiles * P.n_orig;
        const int lag_idx = (int)(item / per_lag);
        const long long rem = item - (long long)lag_idx * per_lag;
        const int itile = (int)(rem / P.n_orig);
        const int k = (int)(rem - (long long)itile * P.n_orig);
        if (lag_idx != cur_lag || since >= flush_every) {
            if (cur_lag >= 0) flush(hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
            cur_lag = lag_idx;
            since = 0;
        }
        ++since;
        const long long fo = P.primo + (long long)k * P.skip;
        const long long fl = fo + (long long)lag_idx * P.every;
        double box[9];
        for (int q = 0; q < 9; ++q)
            box[q] = q < P.box_stride ? P.box[fo * P.box_stride + q] : 0.0;
        double xi[R], yi[R], zi[R];
        int ti[R], ia[R];
        bool vi[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            ia[r] = itile * TI + r * NT + tid;
            vi[r] = ia[r] < P.N;
            const int a = vi[r] ? ia[r] : 0;
            const double *p = P.pos + (fo * N + a) * 3;
            xi[r] = p[0]; yi[r] = p[1]; zi[r] = p[2];
            ti[r] = P.types[a];
            // the caller's ids index the channel table: one out of 0..ntypes-1
            // is reported and its pairs are skipped
            if (vi[r] && (unsigned)ti[r] >= (unsigned)P.ntypes) {
                atomicOr(err, ERR_TYPE_ID);
                vi[r] = false;
            }
        }
        for (int jbase = 0; jbase < P.N; jbase += TJ) {
            const int tj = min(TJ, P.N - jbase);
            __syncthreads();
            for (int q = tid; q < tj; q += NT) {
                const double *p = P.pos + (fl * N + jbase + q) * 3;
                jx[q] = p[0]; jy[q] = p[1]; jz[q] = p[2];
                int t = P.types[jbase + q];
                if ((unsigned)t >= (unsigned)P.ntypes) {
                    atomicOr(err, ERR_TYPE_ID);
                    t = -1;
                }
                jt[q] = t;
            }
            __syncthreads();
            for (int jj = 0; jj < tj; ++jj) {
                const double x = jx[jj], y = jy[jj], z = jz[jj];
                const int tj_ = jt[jj];
                if (tj_ < 0) continue;  // an invalid id (reported above)
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (!vi[r]) continue;
                    const double d2 = ref_d2<TRI>(xi[r], yi[r], zi[r], x, y, z, box, err);
                    const int b = ref_bin(d2, P.rmin, P.dr, P.rmin2, P.rmax2, P.nbin);
                    if (b >= 0) {
                        const int ch =
                            chtab[ti[r] * P.ntypes + tj_] + (ia[r] == jbase + jj ? half : 0);
                        atomicAdd(hist + ch * P.nbin + b, 1u);
                    }
                }
            }
        }
    }
    if (cur_lag >= 0) flush(hist, hlen, P.counts + (long long)cur_lag * P.every * hlen);
}

std::mutex g_setup_mutex;
void *g_scratch_ptr[MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on the current device, resolved once
// per device with that device current.
int scratch_on_current_device(unsigned char **out, int *dev_out, char *msg, size_t msglen)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        snprintf(msg, msglen, "no usable current CUDA device (%s)", cudaGetErrorString(e));
        return GOFR_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            snprintf(msg, msglen, "cudaGetSymbolAddress of the scratch array failed: %s",
                     cudaGetErrorString(e));
            return GOFR_ERR_CUDA;
        }
        g_scratch_ptr[dev] = ptr;
    }
    *out = static_cast<unsigned char *>(g_scratch_ptr[dev]);
    *dev_out = dev;
    return GOFR_OK;
}

}  // namespace noalloc
}  // namespace gofr

extern "C" int gofr_run_f64_noalloc(const double *d_positions, const double *d_boxes,
                                    int box_kind, const int *d_type_ids, unsigned ntypes,
                                    size_t natoms, size_t nframes, const gofr_params *p,
                                    unsigned long long *d_counts, void *stream, char *errbuf,
                                    size_t errlen)
{
    using namespace gofr::noalloc;
    char local[256];
    char *msg = (errbuf && errlen) ? errbuf : local;
    const size_t msglen = (errbuf && errlen) ? errlen : sizeof local;
    msg[0] = '\0';
    if (!d_positions || !d_boxes || !d_type_ids || !d_counts || !p) {
        snprintf(msg, msglen, "null pointer argument");
        return GOFR_ERR_ARG;
    }
    if (box_kind != GOFR_BOX_ORTHO && box_kind != GOFR_BOX_TRICLINIC) {
        snprintf(msg, msglen, "invalid box kind %d", box_kind);
        return GOFR_ERR_ARG;
    }
    if (natoms == 0 || nframes == 0 || natoms > (size_t)(1 << 30)) {
        snprintf(msg, msglen, "natoms must be in 1..2^30 and nframes >= 1");
        return GOFR_ERR_ARG;
    }
    if (ntypes == 0 || ntypes > (unsigned)MAX_TYPES) {
        snprintf(msg, msglen,
                 "ntypes=%u: the allocation-free entry point supports 1..%d types (its channel "
                 "table lives in a fixed %d-byte scratch array)", ntypes, MAX_TYPES,
                 SCRATCH_BYTES);
        return GOFR_ERR_ARG;
    }
    if (p->nbin == 0) {
        snprintf(msg, msglen, "nbin must be > 0");
        return GOFR_ERR_ARG;
    }
    if (p->nparts > 1) {
        snprintf(msg, msglen, "per-partition counts (nparts > 1) need gofr_run");
        return GOFR_ERR_UNSUPPORTED;
    }
    const unsigned skip = p->skip ? p->skip : 1, every = p->every ? p->every : 1;
    const unsigned leff = (p->ntimesteps < p->tmax || p->tmax == 0) ? p->ntimesteps : p->tmax;
    if ((unsigned long long)leff + p->ntimesteps + p->primo > (unsigned long long)nframes + 1) {
        snprintf(msg, msglen,
                 "trajectory is too short for this kind of calculation. Select a different "
                 "starting timestep or lower the size of the average or the lenght of the time "
                 "lag");
        return GOFR_ERR_RANGE;
    }
    const int nch = (int)(ntypes * (ntypes + 1));
    const size_t smem = (size_t)TJ * (3 * 8 + 4) + (size_t)nch * p->nbin * 4 +
                        (size_t)ntypes * ntypes * 2;
    const size_t smem_al = (smem + 127) / 128 * 128;
    unsigned char *scratch = nullptr;
    int dev = -1;
    int rc = scratch_on_current_device(&scratch, &dev, msg, msglen);
    if (rc) return rc;
    int max_smem = 0, sms = 0;
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (smem_al > (size_t)max_smem) {
        snprintf(msg, msglen, "histogram of %d channels x %u bins does not fit in shared memory",
                 nch, p->nbin);
        return GOFR_ERR_UNSUPPORTED;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t n_out = (size_t)leff * nch * p->nbin;

    // channel table of the type pairs (lib/include/gofrt.h:86-104), on the stack
    unsigned short tab[MAX_TYPES * MAX_TYPES];
    for (unsigned a = 0; a < ntypes; ++a)
        for (unsigned c = 0; c < ntypes; ++c) {
            unsigned t1 = a < c ? a : c, t2 = a < c ? c : a;
            tab[a * ntypes + c] =
                (unsigned short)(ntypes * (ntypes + 1) / 2 - (t2 + 1) * (t2 + 2) / 2 + t1);
        }
    // every call shares the scratch: clear the error word, rewrite the table
    cudaError_t e = cudaMemsetAsync(scratch + OFF_ERR, 0, sizeof(unsigned), s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(scratch + OFF_CHTAB, tab, ntypes * ntypes * sizeof(unsigned short),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_counts, 0, n_out * sizeof(unsigned long long), s);
    if (e != cudaSuccess) {
        snprintf(msg, msglen, "CUDA call failed: %s", cudaGetErrorString(e));
        return GOFR_ERR_CUDA;
    }
    const unsigned n_lags = (leff + every - 1) / every;
    const unsigned n_orig = (p->ntimesteps + skip - 1) / skip;
    if (n_lags > 0 && n_orig > 0) {
        Launch L{};
        L.pos = d_positions;
        L.box = d_boxes;
        L.box_stride = box_kind == GOFR_BOX_TRICLINIC ? 9 : 6;
        L.types = d_type_ids;
        L.counts = d_counts;
        L.scratch = scratch;
        L.N = (int)natoms;
        L.nbin = (int)p->nbin;
        L.nch = nch;
        L.ntypes = (int)ntypes;
        L.n_lags = (int)n_lags;
        L.every = (int)every;
        L.n_orig = (int)n_orig;
        L.skip = (int)skip;
        L.primo = (long long)p->primo;
        L.n_itiles = (int)((natoms + TI - 1) / TI);
        L.n_items = (long long)L.n_lags * L.n_itiles * L.n_orig;
        L.dr = (p->rmax - p->rmin) / p->nbin;
        L.rmin = p->rmin;
        L.rmin2 = p->rmin * p->rmin;
        L.rmax2 = p->rmax * p->rmax;
        const bool tri = box_kind == GOFR_BOX_TRICLINIC;
        auto kern = tri ? k_pairs_f64_noalloc<true> : k_pairs_f64_noalloc<false>;
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_al);
        int per_sm = 0;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem_al);
        if (e == cudaSuccess) {
            long long grid = (long long)sms * (per_sm > 0 ? per_sm : 1);
            if (grid > L.n_items) grid = L.n_items;
            kern<<<(unsigned)grid, NT, smem_al, s>>>(L);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) {
            snprintf(msg, msglen, "kernel launch failed: %s", cudaGetErrorString(e));
            return GOFR_ERR_CUDA;
        }
    }
    unsigned errword = 0;
    e = cudaMemcpyAsync(&errword, scratch + OFF_ERR, sizeof errword, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        snprintf(msg, msglen, "CUDA error: %s", cudaGetErrorString(e));
        return GOFR_ERR_CUDA;
    }
    if (errword) {
        snprintf(msg, msglen, "kernel reported error word 0x%x (%s%s)", errword,
                 (errword & ERR_TYPE_ID) ? "a type id outside 0..ntypes-1; its pairs were "
                                           "skipped " : "",
                 (errword & gofr::ERRW_WRAP_LOOP) ? "minimum-image iteration cap" : "");
        return GOFR_ERR_DEVICE;
    }
    return GOFR_OK;
}
