// Warp-streamed cell-list form of the FP32 + FP64-recheck pair kernel.
//
// The reference evaluates all N^2 ordered pairs of every (lag, origin)
// (lib/src/gofrt.cpp:101-102).  As in the block cell-list kernel
// (gofr_cells.cu), the atoms of every frame are binned into cells of edge
// >= rmax / reach and sorted by cell, so a pair the reference counts lies in
// cells at most `reach` apart on every axis; here the unit of neighbourhood
// is much smaller: each WARP owns a small block of cells and streams only
// that block's own neighbourhood, so the pairs evaluated per first atom
// shrink from the neighbourhood of a CTA-sized block to the neighbourhood of
// a warp-sized one.
//
// Lanes hold neighbours, not first atoms: a chunk buffer holds 128 records
// of the neighbourhood (rows packed back to back, several per chunk when
// they are short), each lane keeps four of them in registers, and the warp
// walks the block's first atoms one at a time, each broadcast
// from shared memory, so no lane idles for want of a first atom whatever the
// block's atom count (only the last chunk of a neighbourhood is partly
// padding).
//
// Layout per frame (built once per upload and grid): records
// {x, y, z, type << 24 | atom id} (float4, the coordinates wrapped into the
// box in FP64 and rounded to FP32 about the box centre, exactly as the block
// kernel's), sorted by cell, x fastest; cell start offsets.  A row of cells
// of a neighbourhood is one contiguous run of 16-byte records, so a warp
// stages it into shared memory with one 1-D bulk copy (TMA, cp.async.bulk)
// per piece (a row's run of records, or the part of it that fits), up to
// MAXP pieces and CH records per chunk, two chunk buffers per warp,
// completion tracked by one mbarrier per buffer.  Cells reached across the
// box boundary are the periodic image of the cell: after the copy lands,
// each lane moves its records to their piece's image (x += fl32 of the
// lattice vector, one FP32 rounding per axis; orthorhombic: s fl32(L), the
// block kernel's arithmetic), so the pair arithmetic and its certified error
// bound (gofr_capi.cu, error_bound_cells) are the block kernel's.
//
// Triclinic boxes (upper-triangular cell vectors a, b, c) use the same
// kernel.  The reference's minimum image (z, then y, then x) leaves every
// component within half the box edge, so its image of a pair is the one
// lattice translate inside the axis-aligned box [-L/2, L/2]^3, and a pair it
// counts (distance < rmax < L/2) has exactly one image within rmax.  Cells
// are therefore an axis-aligned grid of the cell's axis-aligned fundamental
// domain, atoms reduced into it by the lattice; a layer reached across a z
// face is the image +-c, shifted in y and x by the tilts, and a row reached
// across a y face the image +-b, shifted in x: each layer's rows and each
// row's cells start a fraction of a cell off, which host tables give (one
// more cell where the shift is not whole), together with the FP32 lattice
// vector of each image.
//
// Warps never wait for one another inside a work item (lag, origin, part of
// the warp blocks): they pull warp blocks from a shared counter, stream
// their own neighbourhoods and add their candidates to the CTA's shared
// histogram; the CTA synchronises only at the end of the item, to add the
// histogram to the counts.  Candidates (FP32 d2 <= hi_f) are compacted into
// a dense per-warp queue as they are found (one ballot per first atom and
// record slot: each candidate lane writes at the warp's count plus the
// candidates of the lanes below it); an entry names the first atom and the
// record of the current chunk buffer, 16 bits.  The queue is binned 32
// entries at a time, every lane busy: when it is nearly full and at the end
// of each chunk (before the buffer is refilled), d2 recomputed with the
// pair loop's arithmetic (the same value), then the block kernel's
// certified window test and predicated shared-memory reductions.
#include <cstdint>
#include <cuda_runtime.h>

#include "gofr_device.cuh"
#include "gofr_internal.h"

namespace gofr {
namespace cellw {

constexpr int CH = 128;        // neighbour records per chunk buffer: 4 per lane
constexpr int MAXP = 8;        // pieces (bulk copies) per chunk
constexpr int FA = 64;         // first atoms per batch
constexpr int CQ = 1024;       // candidate queue entries of a warp
constexpr int CQ_ROOM = 4 * 32; // entries one first atom can add (4 records x 32 lanes)
constexpr int QW = 32;         // FP64 recheck queue of a warp
constexpr int MAXROWS = CELLW_MAX_ROWS;  // neighbourhood rows of a warp block
static_assert(CH == 4 * 32, "four records per lane");
static_assert(CQ / 32 <= 32, "one bit per binning round in a 32-bit recheck mask");
static_assert(CH <= 256 && FA <= 256, "a queue entry names a first atom and a record in 8 bits each");

// floor(a / n) for n > 0
__device__ __forceinline__ int floordiv(int a, int n) { return a >= 0 ? a / n : -((n - 1 - a) / n); }

constexpr unsigned SEG_BEGIN = 0x1ffffffu;  // a segment's begin; its image index above bit 25

// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) writes to the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Shared memory of one warp.
struct WarpArea {
    float4 buf[2][CH];           // chunk buffers (bulk-copy destinations, 16-byte aligned)
    float4 fi[FA];               // first atoms of the batch {x, y, z, type << 24 | id}
    unsigned short cq[CQ];       // candidate queue: first atom << 8 | record of the current chunk
    uint4 q[QW];                 // FP64 recheck queue {ia, ja, channel, 0}
    int2 seg[2 * MAXROWS];       // sorted ranges of the neighbourhood rows (two halves each):
                                 // {begin | image << 25, end}
    int4 pc[2][MAXP];            // pieces of each buffer {first record, source record, count, image}
    uint64_t bar[2];             // one mbarrier per chunk buffer
    int n[2];                    // records in each buffer
    int np[2];                   // pieces in each buffer
    int qn;                      // entries in q
    int pad[3];
};

// Chunk walker state (the same values in every lane of a warp).
struct Walk {
    int row, half, off;          // current segment (row, half) and offset into it
};

// NWARP warps per CTA (8: two CTAs per SM, 16: one), HCOPY copies of the
// shared histogram (warp w adds to copy w HCOPY / NWARP: the privatisation
// depth, fewer warps contending for each bin).
template <int NWARP, int HCOPY>
__global__ void __launch_bounds__(NWARP * 32, 16 / NWARP) k_pairs_cellw(const CellwLaunch C,
                                                                        int win_cap, int hist_cap)
{
    constexpr int NT = NWARP * 32;
    extern __shared__ __align__(128) unsigned char smem[];
    WarpArea *const areas = reinterpret_cast<WarpArea *>(smem);
    float2 *const win = reinterpret_cast<float2 *>(areas + NWARP);
    unsigned *const hist = reinterpret_cast<unsigned *>(win + win_cap);
    unsigned short *const chtab = reinterpret_cast<unsigned short *>(hist + HCOPY * hist_cap);
    __shared__ int s_next, s_abort;
    __shared__ unsigned long long s_pairs;  // pairs evaluated in the current item
    __shared__ float4 s_shift[CELLW_NSHIFT];
    __shared__ int2 s_ny[3], s_nx[15];

    const PairLaunch &P = C.pair;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;  // the lanes below this one
    WarpArea &A = areas[warp];
    const int hlen = P.nch * P.nbin;
    unsigned *const whist = hist + (warp * HCOPY / NWARP) * hist_cap;  // this warp's copy
    const int half_ch = P.nch / 2;
    const float hi_f = P.hi_f;
    const int ncx = C.nc[0], ncy = C.nc[1], ncz = C.nc[2];
    const int ncell = ncx * ncy * ncz;
    const int nwx = C.nw[0], nwy = C.nw[1], nwz = C.nw[2];
    const int nwb = nwx * nwy * nwz;
    const long long NP = P.NP;

    for (int i = tid; i < P.nbin; i += NT) win[i] = P.win[i];
    for (int c = 0; c < HCOPY; ++c)
        for (int i = tid; i < hlen; i += NT) hist[c * hist_cap + i] = 0u;
    for (int i = tid; i < P.ntypes * P.ntypes; i += NT) chtab[i] = P.chtab[i];
    for (int i = tid; i < CELLW_NSHIFT; i += NT) s_shift[i] = C.shift[i];
    if (tid < 3) s_ny[tid] = make_int2(C.ny_lo[tid], C.ny_hi[tid]);
    if (tid < 15) s_nx[tid] = make_int2(C.nx_lo[tid], C.nx_hi[tid]);
    if (lane == 0) {
        mbar_init(&A.bar[0], 1);
        mbar_init(&A.bar[1], 1);
        A.qn = 0;
        fence_mbar_init();
    }
    if (tid == 0) s_abort = 0;
    __syncthreads();

    unsigned ph0 = 0u, ph1 = 0u;      // mbarrier phases of the two buffers
    bool dead = false;                // a bounded wait of this warp ran out
    unsigned long long n_cand = 0, n_rech = 0, n_eval = 0;

    for (long long g = blockIdx.x; g < P.n_items; g += gridDim.x) {
        // item = (lag, origin, part): lag slowest
        const long long per_lag = (long long)P.n_orig * C.parts;
        const int lag_idx = (int)(g / per_lag);
        const long long rem = g - (long long)lag_idx * per_lag;
        const int k = (int)(rem / C.parts);
        const int part = (int)(rem - (long long)k * C.parts);
        const int wb0 = (int)((long long)part * nwb / C.parts);
        const int wb1 = (int)((long long)(part + 1) * nwb / C.parts);
        const long long fo = P.primo + (long long)k * P.skip;
        const long long fl = fo + (long long)lag_idx * P.every;
        const int *st_o = C.start + fo * (long long)(ncell + 1);
        const int *st_l = C.start + fl * (long long)(ncell + 1);
        const float4 *rec_o = C.wpos + fo * NP;
        const float4 *rec_l = C.wpos + fl * NP;
        if (tid == 0) {
            s_next = wb0;
            s_pairs = 0ull;
        }
        __syncthreads();

        // the reference's d2 of a pair in FP64 (its minimum image for the box kind)
        auto ref_d2_box = [&](const double *xi64, const double *xj64, const double *box) {
            return P.tric ? ref_d2<true>(xi64[0], xi64[1], xi64[2], xj64[0], xj64[1], xj64[2],
                                         box, P.err)
                          : ref_d2<false>(xi64[0], xi64[1], xi64[2], xj64[0], xj64[1], xj64[2],
                                          box, P.err);
        };
        // Bins the warp's queued candidates 32 at a time.  An entry's FP32 d2
        // is recomputed from the first atom and the chunk buffer's record
        // with the pair loop's operations (one difference per axis, a
        // multiply, two FMAs: the same value); pairs outside their bin's
        // certified window are flagged per round and recomputed in FP64
        // after the rounds.
        int cn = 0;  // entries in the queue (the same in every lane)
        auto flush_q = [&](const float4 *bufp) {
            __syncwarp();  // every lane's entries and first atoms visible
            unsigned needm = 0u;  // rounds whose entry of this lane goes to the recheck
            // each round's entry, first atom and record are loaded a round ahead
            // (a lane past the queue's end reads entry 0's: valid addresses, unused)
            bool vn = lane < cn;
            unsigned en = vn ? (unsigned)A.cq[lane] : 0u;
            float4 fin = A.fi[en >> 8], fjn = bufp[en & 0xffu];
            for (int g0 = 0; g0 < cn; g0 += 32) {
                const bool v = vn;
                const float4 fi = fin, fj = fjn;
                vn = g0 + 32 + lane < cn;
                en = vn ? (unsigned)A.cq[g0 + 32 + lane] : 0u;
                fin = A.fi[en >> 8];
                fjn = bufp[en & 0xffu];
                const float dx = __fsub_rn(fi.x, fj.x), dy = __fsub_rn(fi.y, fj.y),
                            dz = __fsub_rn(fi.z, fj.z);
                float d2 = __fmul_rn(dx, dx);
                d2 = __fmaf_rn(dy, dy, d2);
                d2 = __fmaf_rn(dz, dz, d2);
                const unsigned iv = __float_as_uint(fi.w), jv = __float_as_uint(fj.w);
                const int ch = chtab[(int)(iv >> 24) * P.ntypes + (int)(jv >> 24)] +
                               (((iv ^ jv) & 0xffffffu) == 0u ? half_ch : 0);
                // bin guess (the window test decides): (sqrt(d2) - rmin) / dr as one
                // FMA, negative guesses clamped to the last bin (whose window fails)
                const int b_ = __float2int_rd(
                    __fmaf_rn(sqrt_guess(d2), P.inv_dr_f, -P.rmin_f * P.inv_dr_f));
                const int bi = (int)min((unsigned)b_, (unsigned)(P.nbin - 1));
                const float2 w = win[bi];
                const bool test = v && d2 >= P.lo_f;
                const bool inw = d2 >= w.x && d2 <= w.y;
                red_shared_add1_if(smem_u32(whist + ch * P.nbin + bi),
                                   test && inw &&
                                       GOFR_CHECK(ch >= 0 && ch < P.nch && bi >= 0 && bi < P.nbin,
                                                  P.err));
                needm |= (test && !inw) ? 1u << (g0 >> 5) : 0u;
            }
            if (__any_sync(0xffffffffu, needm != 0u)) {
                while (needm) {
                    const int it = __ffs(needm) - 1;
                    needm &= needm - 1u;
                    const unsigned e = A.cq[it * 32 + lane];
                    const unsigned iv = __float_as_uint(A.fi[e >> 8].w),
                                   jv = __float_as_uint(bufp[e & 0xffu].w);
                    const int ia = (int)(iv & 0xffffffu), ja = (int)(jv & 0xffffffu);
                    const int ch = chtab[(int)(iv >> 24) * P.ntypes + (int)(jv >> 24)] +
                                   (ia == ja ? half_ch : 0);
                    ++n_rech;
                    const int slot = atomicAdd(&A.qn, 1);
                    if (slot < QW) {
                        A.q[slot] = make_uint4((unsigned)ia, (unsigned)ja, (unsigned)ch, 0u);
                    } else {
                        const double *xi64 = P.pos64 + (fo * P.N + ia) * 3;
                        const double *xj64 = P.pos64 + (fl * P.N + ja) * 3;
                        const double d2d = ref_d2_box(xi64, xj64, P.box64 + fo * 9);
                        const int bb = ref_bin(d2d, P.rmin, P.dr, P.rmin2, P.rmax2, P.nbin);
                        if (bb >= 0) atomicAdd(whist + ch * P.nbin + bb, 1u);
                    }
                }
            }
            if (lane == 0) n_cand += (unsigned)cn;
            cn = 0;
            __syncwarp();  // every lane done with the entries before they are rewritten
        };
        // Recomputes the warp's queued pairs in exact FP64 (reference arithmetic).
        auto drain_queue = [&]() {
            __syncwarp();
            const int nq = min(A.qn, QW);
            for (int q = lane; q < nq; q += 32) {
                const uint4 e = A.q[q];
                const double *xi64 = P.pos64 + (fo * P.N + (int)e.x) * 3;
                const double *xj64 = P.pos64 + (fl * P.N + (int)e.y) * 3;
                const double d2d = ref_d2_box(xi64, xj64, P.box64 + fo * 9);
                const int bb = ref_bin(d2d, P.rmin, P.dr, P.rmin2, P.rmax2, P.nbin);
                if (bb >= 0) atomicAdd(whist + (int)e.z * P.nbin + bb, 1u);
            }
            __syncwarp();
            if (lane == 0) A.qn = 0;
            __syncwarp();
        };

        while (!dead) {
            int wb = 0;
            if (lane == 0) wb = atomicAdd(&s_next, 1);
            wb = __shfl_sync(0xffffffffu, wb, 0);
            if (wb >= wb1) break;
            const int wz = wb / (nwx * nwy), wy = (wb / nwx) % nwy, wx = wb % nwx;
            const int cx0 = wx * C.w[0], cy0 = wy * C.w[1], cz0 = wz * C.w[2];
            const int cnx = min(C.w[0], ncx - cx0), cny = min(C.w[1], ncy - cy0),
                      cnz = min(C.w[2], ncz - cz0);
            // rows of the warp block (w_y w_z <= 16 of them): lane r holds row
            // r's range and the inclusive prefix of the row lengths
            const int nir = cny * cnz;
            int ib = 0, ilen = 0;
            if (lane < nir) {
                const int ry = lane % cny, rz = lane / cny;
                const int base = ((cz0 + rz) * ncy + (cy0 + ry)) * ncx + cx0;
                ib = st_o[base];
                ilen = st_o[base + cnx] - ib;
            }
            int ipre = ilen;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, ipre, o);
                if (lane >= o) ipre += v;
            }
            const int n_i = __shfl_sync(0xffffffffu, ipre, 31);
            if (n_i == 0) continue;
            // the neighbourhood: layers uz (image sz), in each the rows uy
            // (image sy), each row the cells ux in one or two sorted ranges
            // (two when the row wraps the box: images sx and sx + 1); the
            // layer's row slots beyond its own rows stay empty
            const int jny = cny + C.ny_span;
            const int nrows = (cnz + C.nz_hi - C.nz_lo + 1) * jny;
            for (int rr = lane; rr < nrows; rr += 32) {
                const int lz = rr / jny, k = rr - lz * jny;
                const int uz = cz0 + C.nz_lo + lz;
                const int sz = floordiv(uz, ncz), cz = uz - sz * ncz;
                int2 s0 = make_int2(0, 0), s1 = make_int2(0, 0);
                // the host keeps every image reached inside the tables and every
                // row within one wrap of the box; a row outside them is reported
                // and left empty (no access outside the tables or the frame)
                bool ok = sz >= -1 && sz <= 1;
                const int2 yr = ok ? s_ny[sz + 1] : make_int2(0, -1 - cny);
                if (k <= cny + yr.y - yr.x) {
                    const int uy = cy0 + yr.x + k;
                    const int sy = floordiv(uy, ncy), cy = uy - sy * ncy;
                    ok = sy >= -2 && sy <= 2;
                    const int2 xr = ok ? s_nx[(sz + 1) * 5 + sy + 2] : make_int2(0, 0);
                    const int ux = cx0 + xr.x, len = cnx + xr.y - xr.x + 1;
                    const int sx = floordiv(ux, ncx), a = ux - sx * ncx, b = a + len;
                    ok = ok && sx >= -2 && len >= 0 && len <= ncx && (b <= ncx ? sx <= 2 : sx <= 1);
                    if (ok) {
                        const int base = (cz * ncy + cy) * ncx;
                        const unsigned code =
                            (unsigned)((sx + 2) + 5 * (sy + 2) + 25 * (sz + 1)) << 25;
                        if (b <= ncx) {
                            s0 = make_int2((int)((unsigned)st_l[base + a] | code), st_l[base + b]);
                        } else {
                            s0 = make_int2((int)((unsigned)st_l[base + a] | code),
                                           st_l[base + ncx]);
                            s1 = make_int2((int)((unsigned)st_l[base] | (code + (1u << 25))),
                                           st_l[base + b - ncx]);
                        }
                    }
                }
                if (!ok) atomicOr(P.err, ERRW_BOUNDS);
                A.seg[2 * rr] = s0;
                A.seg[2 * rr + 1] = s1;
            }
            __syncwarp();
            int n_j = 0;
            for (int s = lane; s < 2 * nrows; s += 32)
                n_j += A.seg[s].y - (int)((unsigned)A.seg[s].x & SEG_BEGIN);
            n_j = __reduce_add_sync(0xffffffffu, n_j);
            // Fills buffer b with the next records of the neighbourhood: up to CH
            // records from up to MAXP pieces (every lane walks the segments
            // alike); lane 0 then expects their bytes on the buffer's mbarrier
            // and issues one bulk copy per piece.  False at the end of the
            // neighbourhood (nothing issued).
            auto issue = [&](Walk &w, int b) -> bool {
                int filled = 0, np = 0;
                while (w.row < nrows && filled < CH && np < MAXP) {
                    const int2 sg = A.seg[2 * w.row + w.half];
                    const int beg = (int)((unsigned)sg.x & SEG_BEGIN);
                    const int len = sg.y - beg;
                    if (w.off < len) {
                        const int n = min(CH - filled, len - w.off);
                        if (lane == 0)
                            A.pc[b][np] = make_int4(filled, beg + w.off, n,
                                                    (int)((unsigned)sg.x >> 25));
                        ++np;
                        filled += n;
                        w.off += n;
                        continue;
                    }
                    w.off = 0;
                    if (++w.half == 2) { w.half = 0; ++w.row; }
                }
                if (filled == 0) return false;
                if (lane == 0) {
                    A.n[b] = filled;
                    A.np[b] = np;
                    mbar_arrive_expect_tx(&A.bar[b], (unsigned)(filled * 16));
                    for (int p = 0; p < np; ++p) {
                        const int4 pc = A.pc[b][p];
                        bulk_g2s(&A.buf[b][pc.x], rec_l + pc.y, (unsigned)(pc.z * 16), &A.bar[b]);
                    }
                }
                return true;
            };

            for (int ibase = 0; ibase < n_i && !dead; ibase += FA) {
                // first atoms ibase .. ibase + na - 1 of the block
                const int na = min(FA, n_i - ibase);
                for (int q0 = 0; q0 < na; q0 += 32) {
                    const int q = q0 + lane;
                    // row of atom ibase + q (every lane takes part in the shuffles)
                    const int qq = min(ibase + q, n_i - 1);
                    int row = 0;
                    for (int rr = 0; rr < nir; ++rr)
                        row += (qq >= __shfl_sync(0xffffffffu, ipre, rr)) ? 1 : 0;
                    const int rb = __shfl_sync(0xffffffffu, ib, row);
                    const int rp = __shfl_sync(0xffffffffu, ipre - ilen, row);
                    if (q < na) A.fi[q] = rec_o[rb + (qq - rp)];
                }
                if (lane == 0) {
                    const unsigned long long pe = (unsigned long long)na * (unsigned long long)n_j;
                    n_eval += pe;
                    atomicAdd(&s_pairs, pe);
                }
                // earlier generic accesses of both buffers (records moved to their
                // image, padding, reads) before the bulk copies that refill them
                fence_proxy_async_smem();
                __syncwarp();
                Walk w{0, 0, 0};
                bool have0 = issue(w, 0);
                bool have1 = have0 && issue(w, 1);
                for (int c = 0; (c & 1) ? have1 : have0; ++c) {
                    const int b = c & 1;
                    const bool ok = mbar_wait_bounded(&A.bar[b], b ? ph1 : ph0);
                    if (!__all_sync(0xffffffffu, ok)) {
                        // give the other buffer's copy a bounded chance to land,
                        // then stop this warp's work (the CTA ends at the item)
                        if (lane == 0 && (b ? have0 : have1))
                            mbar_wait_bounded(&A.bar[b ^ 1], b ? ph0 : ph1);
                        if (lane == 0) {
                            atomicOr(P.err, ERRW_WAIT_TIMEOUT);
                            s_abort = 1;
                        }
                        dead = true;
                        break;
                    }
                    if (b) ph1 ^= 1u; else ph0 ^= 1u;
                    const int n = A.n[b], np = A.np[b];
                    float4 *const bufp = A.buf[b];
                    // this lane's records lane + 32 t (consecutive lanes, consecutive
                    // records: no bank conflict): moved to their piece's image
                    // (image (0, 0, 0) adds zeros: x + 0 = x) and written back for
                    // the binning; records past n are NaN (never a candidate)
                    float rx[4], ry[4], rz[4];
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const int k = lane + 32 * t;
                        float4 v = make_float4(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000),
                                               __int_as_float(0x7fc00000),
                                               __uint_as_float(0xffffffffu));
                        if (k < n) {
                            int code = A.pc[b][0].w;
                            for (int p = 1; p < np; ++p) {
                                const int4 pc = A.pc[b][p];
                                if (pc.x <= k) code = pc.w;
                            }
                            const float4 sh = s_shift[code];
                            v = bufp[k];
                            v.x = __fadd_rn(v.x, sh.x);
                            v.y = __fadd_rn(v.y, sh.y);
                            v.z = __fadd_rn(v.z, sh.z);
                        }
                        bufp[k] = v;
                        rx[t] = v.x; ry[t] = v.y; rz[t] = v.z;
                    }
                    __syncwarp();
                    const unsigned eb0 = (unsigned)lane;
                    for (int i = 0; i < na; ++i) {
                        // first atom i (broadcast) against this lane's four records
                        const float4 fv = A.fi[i];
                        float dd[4];
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            // one difference per axis, a multiply, two FMAs (the
                            // binning recomputes d2 with the same operations)
                            const float ex = __fsub_rn(fv.x, rx[t]), ey = __fsub_rn(fv.y, ry[t]),
                                        ez = __fsub_rn(fv.z, rz[t]);
                            float s2 = __fmul_rn(ex, ex);
                            s2 = __fmaf_rn(ey, ey, s2);
                            dd[t] = __fmaf_rn(ez, ez, s2);
                        }
                        const float d0 = dd[0], d1 = dd[1], d2v = dd[2], d3 = dd[3];
                        // entries i << 8 | record, compacted by one ballot per record slot
                        const unsigned eb = (unsigned)i << 8 | eb0;
                        const bool p0 = d0 <= hi_f, p1 = d1 <= hi_f, p2 = d2v <= hi_f,
                                   p3 = d3 <= hi_f;
                        const unsigned b0 = __ballot_sync(0xffffffffu, p0),
                                       b1 = __ballot_sync(0xffffffffu, p1),
                                       b2 = __ballot_sync(0xffffffffu, p2),
                                       b3 = __ballot_sync(0xffffffffu, p3);
                        const int c1 = cn + __popc(b0), c2 = c1 + __popc(b1),
                                  c3 = c2 + __popc(b2);
                        if (p0) A.cq[cn + __popc(b0 & lt)] = (unsigned short)eb;
                        if (p1) A.cq[c1 + __popc(b1 & lt)] = (unsigned short)(eb + 32u);
                        if (p2) A.cq[c2 + __popc(b2 & lt)] = (unsigned short)(eb + 64u);
                        if (p3) A.cq[c3 + __popc(b3 & lt)] = (unsigned short)(eb + 96u);
                        cn = c3 + __popc(b3);
                        if (!GOFR_CHECK(cn <= CQ, P.err)) cn = CQ;
                        // room for the next first atom's entries
                        if (cn > CQ - CQ_ROOM) flush_q(bufp);
                    }
                    // the entries name records of this buffer: bin them before it is refilled
                    if (cn > 0) flush_q(bufp);
                    fence_proxy_async_smem();
                    __syncwarp();  // every lane done with buffer b
                    if (b) have1 = issue(w, 1);
                    else have0 = issue(w, 0);
                }
                if (A.qn > QW / 2) drain_queue();
            }
        }
        if (!dead) drain_queue();
        __syncthreads();  // every warp done with this item
        // a u32 shared bin holds the item's hits exactly only while the item
        // evaluated fewer than 2^32 pairs (the host sizes items far below)
        if (tid == 0 && s_pairs > 0xffffffffull) {
            atomicOr(P.err, ERRW_HIST_OVERFLOW);
            s_abort = 1;
        }
        __syncthreads();
        const bool abort = s_abort != 0;
        // add the item's histogram copies to its lag's counts, then clear them
        for (int i = tid; i < hlen; i += NT) {
            unsigned long long v = 0;
#pragma unroll
            for (int c = 0; c < HCOPY; ++c) {
                v += hist[c * hist_cap + i];
                hist[c * hist_cap + i] = 0u;
            }
            if (v && !abort)
                atomicAdd(P.counts + (long long)lag_idx * P.every * hlen + i, v);
        }
        __syncthreads();
        if (abort) break;
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_cand += __shfl_xor_sync(0xffffffffu, n_cand, o);
        n_rech += __shfl_xor_sync(0xffffffffu, n_rech, o);
        n_eval += __shfl_xor_sync(0xffffffffu, n_eval, o);
    }
    if (lane == 0) {
        if (n_cand) atomicAdd(P.stats + ST_CANDIDATES, n_cand);
        if (n_rech) atomicAdd(P.stats + ST_RECHECKS, n_rech);
        if (n_eval) atomicAdd(P.stats + ST_EVALUATED, n_eval);
    }
}

}  // namespace cellw

int cellw_smem_bytes(int nch, int nbin, int ntypes, int cta_warps, int hcopy)
{
    using namespace cellw;
    size_t b = sizeof(WarpArea) * cta_warps + (size_t)nbin * 8 +
               (size_t)hcopy * nch * nbin * 4 + (size_t)ntypes * ntypes * 2;
    return (int)((b + 127) / 128 * 128);
}

int cellw_chunk_records() { return cellw::CH; }
int cellw_batch_atoms() { return cellw::FA; }
int cellw_chunk_pieces() { return cellw::MAXP; }

// Sorted AoS copy of every frame: {x, y, z, type << 24 | id} with the block
// kernel's coordinates (w = x - n L, n = floor((x - xlo) / L), one FMA in
// FP64, then fl32(fl64(w - c)), c the box centre); triclinic: w the lattice
// reduction of wrap_tric64, the same FP32 rounding about the centre.
__global__ void k_cell_scatter_w(const double *__restrict__ pos64,
                                 const unsigned char *__restrict__ types8, size_t T, size_t N,
                                 size_t NP, int ncell, double xlo, double ylo, double zlo,
                                 double Lx, double Ly, double Lz, double xy, double xz, double yz,
                                 int tric, double cx, double cy, double cz,
                                 const int *__restrict__ cell_of, const int *__restrict__ rank_of,
                                 const int *__restrict__ start, float4 *__restrict__ wpos)
{
    const double lo[3] = {xlo, ylo, zlo}, L[3] = {Lx, Ly, Lz}, c[3] = {cx, cy, cz};
    const double tilt[3] = {xy, xz, yz};
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < T * N;
         g += (size_t)gridDim.x * blockDim.x) {
        const size_t f = g / N, a = g - f * N;
        const size_t d = (size_t)start[f * (size_t)(ncell + 1) + cell_of[g]] + rank_of[g];
        const double *p = pos64 + g * 3;
        float v[3];
        if (tric) {
            double w[3];
            wrap_tric64(p, lo, L, tilt, w);
#pragma unroll
            for (int k = 0; k < 3; ++k) v[k] = __double2float_rn(__dsub_rn(w[k], c[k]));
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double n = floor(__ddiv_rn(__dsub_rn(p[k], lo[k]), L[k]));
                const double w = __fma_rn(-n, L[k], p[k]);
                v[k] = __double2float_rn(__dsub_rn(w, c[k]));
            }
        }
        wpos[f * NP + d] =
            make_float4(v[0], v[1], v[2], __uint_as_float(((unsigned)types8[a] << 24) | (unsigned)a));
    }
}

int launch_cell_scatter_w(const double *pos64, const unsigned char *types8, size_t T, size_t N,
                          const double *box_internal, const double *centre, const int *nc,
                          bool tric, const int *cell_of, const int *rank_of, const int *start,
                          float4 *wpos, cudaStream_t s)
{
    const int ncell = nc[0] * nc[1] * nc[2];
    const size_t NP = padded_natoms(N);
    // padding records: NaN coordinates (never read as atoms)
    if (cudaMemsetAsync(wpos, 0xff, T * NP * sizeof(float4), s) != cudaSuccess) return -1;
    const size_t total = T * N;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    const double Lx = 2.0 * box_internal[3], Ly = 2.0 * box_internal[4], Lz = 2.0 * box_internal[5];
    k_cell_scatter_w<<<blocks, 256, 0, s>>>(pos64, types8, T, N, NP, ncell, box_internal[0],
                                            box_internal[1], box_internal[2], Lx, Ly, Lz,
                                            box_internal[6], box_internal[7], box_internal[8],
                                            tric ? 1 : 0, centre[0], centre[1], centre[2],
                                            cell_of, rank_of, start, wpos);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int NWARP, int HCOPY>
static int launch_cellw_shape(const CellwLaunch &C, int num_sms, cudaStream_t s)
{
    using namespace cellw;
    constexpr int NT = NWARP * 32;
    auto kern = k_pairs_cellw<NWARP, HCOPY>;
    const int smem = cellw_smem_bytes(C.pair.nch, C.pair.nbin, C.pair.ntypes, NWARP, HCOPY);
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
        cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem) != cudaSuccess)
        return -1;
    if (per_sm < 1) return -2;
    long long grid = (long long)num_sms * per_sm;
    if (grid > C.pair.n_items) grid = C.pair.n_items;
    kern<<<(unsigned)grid, NT, smem, s>>>(C, C.pair.nbin, C.pair.nch * C.pair.nbin);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_cellw_pairs(const CellwLaunch &C, int num_sms, cudaStream_t s)
{
    if (C.pair.n_items <= 0) return 0;
    if (C.cta_warps == 16) {
        return C.hcopy == 2 ? launch_cellw_shape<16, 2>(C, num_sms, s)
                            : launch_cellw_shape<16, 1>(C, num_sms, s);
    }
    return C.hcopy == 2 ? launch_cellw_shape<8, 2>(C, num_sms, s)
                        : launch_cellw_shape<8, 1>(C, num_sms, s);
}

}  // namespace gofr
