/*
 * CPU restatement of analisi's Gofrt hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker that the GPU kernels of analisi_gb300 are compared
 * against, and the CPU baseline that bench.py times.  Nothing in the product
 * path links or calls it.  It must be compiled with -ffp-contract=off (the
 * build recipe in oracle/oracle.py does so): the reference computes
 * d2 += x*x with a separate multiply and add, and a compiler that fuses them
 * into an FMA (GCC on aarch64 does by default) changes the last bit of d2.
 *
 * Parity of this restatement with the reference itself is pinned by
 * tests/test_oracle_vs_reference.py (run where the reference sources are
 * present; it builds oracle/_ref with oracle/build_ref.sh) and by the fixtures
 * in tests/golden/, which were produced by the reference build.
 *
 * Reference citations (paths inside the analisi project):
 *   lib/src/gofrt.cpp:96-122          Gofrt::calc_single_th   (pair loop, filter, binning)
 *   lib/src/gofrt.cpp:74-93           Gofrt::calc_init        (range check, incr)
 *   lib/src/gofrt.cpp:41-63           Gofrt::reset            (leff, data_length)
 *   lib/src/gofrt.cpp:127-132         Gofrt::calc_end         (thread-buffer fold order)
 *   lib/include/gofrt.h:86-104        Gofrt::get_itype        (type-pair channel)
 *   lib/include/basetrajectory.h:181-219  d2_minImage / d2_minImage_triclinic
 *   lib/include/basetrajectory.h:224-268  minImage_triclinic<TRICLINIC>
 *   lib/include/basetrajectory.h:94-105   lammps_to_internal
 *   lib/include/basetrajectory.h:145-161  pbc_wrap
 *   lib/include/calculatemultithread.h:50-78,80-104,106-162  split + loops
 *   lib/src/msd.cpp:37-118            MSD reset / calc_init / calc_single_th
 *   lib/src/trajectory_numpy.cpp:201-222  calc_cm_pos_vel  (centres of mass)
 *   lib/src/neighbour.cpp:9-97        Neighbours update_neigh / get_sann_n
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

/* Iterative minimum image, z then y then x, strict '>' against the half edge
 * (basetrajectory.h:224-268).  tilt = {xy, xz, yz}; ignored when !tric. */
static void oracle_min_image(double d[3], const double lh[3], const double tilt[3], int tric)
{
    while (fabs(d[2]) > lh[2]) {
        if (d[2] < 0.0) {
            d[2] += lh[2] * 2;
            if (tric) { d[1] += tilt[2]; d[0] += tilt[1]; }
        } else {
            d[2] -= lh[2] * 2;
            if (tric) { d[1] -= tilt[2]; d[0] -= tilt[1]; }
        }
    }
    while (fabs(d[1]) > lh[1]) {
        if (d[1] < 0.0) {
            d[1] += lh[1] * 2;
            if (tric) d[0] += tilt[0];
        } else {
            d[1] -= lh[1] * 2;
            if (tric) d[0] -= tilt[0];
        }
    }
    while (fabs(d[0]) > lh[0]) {
        if (d[0] < 0.0) d[0] += lh[0] * 2;
        else d[0] -= lh[0] * 2;
    }
}

/* Square of the minimum-image distance with the box of the first frame
 * (basetrajectory.h:181-219).  box = internal format
 * {xlo, ylo, zlo, lx/2, ly/2, lz/2, xy, xz, yz}. */
double oracle_d2(const double *xi, const double *xj, const double *box, int tric)
{
    double x[3], d2 = 0.0;
    static const double zero3[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k) x[k] = xi[k] - xj[k];
    oracle_min_image(x, box + 3, tric ? box + 6 : zero3, tric);
    for (int k = 0; k < 3; ++k) d2 += x[k] * x[k];
    return d2;
}

/* Bin of a squared distance, or -1 when the pair is not counted
 * (gofrt.cpp:104,114-118): the filter is on d2 against rmin*rmin and
 * rmax*rmax, the index is floorf of the double quotient converted to float. */
int oracle_bin(double d2, double rmin, double rmax, unsigned nbin)
{
    double dr = (rmax - rmin) / nbin;
    double rmax2 = rmax * rmax, rmin2 = rmin * rmin;
    if (d2 > rmax2 || d2 < rmin2) return -1;
    double d = sqrt(d2);
    float fl = floorf((float)((d - rmin) / dr));
    /* float->int of NaN or of a value beyond int is INT_MIN on x86-64 (the
     * platform the reference goldens come from) and is dropped there; aarch64
     * would give 0 or saturate, so those cases are made explicit here. */
    if (fl != fl || fl >= 2147483648.0f || fl < -2147483648.0f) return -1;
    int idx = (int)fl;
    if ((unsigned)idx < nbin && idx >= 0) return idx;
    return -1;
}

/* Type-pair channel (gofrt.h:86-104). */
unsigned oracle_channel(unsigned t1, unsigned t2, unsigned ntypes)
{
    if (t2 < t1) { unsigned tmp = t2; t2 = t1; t1 = tmp; }
    return ntypes * (ntypes + 1) / 2 - (t2 + 1) * (t2 + 2) / 2 + t1;
}

/* lammps {xlo,xhi,ylo,yhi,zlo,zhi} -> internal {xlo,ylo,zlo,lx/2,ly/2,lz/2}
 * (basetrajectory.h:94-105), in place; tilts in c[6..8] are untouched. */
void oracle_lammps_to_internal(double *c)
{
    double t = c[4];
    c[5] = (c[5] - c[4]) / 2;
    c[4] = (c[3] - c[2]) / 2;
    c[3] = (c[1] - c[0]) / 2;
    c[1] = c[2];
    c[2] = t;
}

/* Wrap every atom of frame idx around the box centre (basetrajectory.h:145-161). */
void oracle_pbc_wrap(double *pos, const double *boxes, size_t box_stride, int tric,
                     size_t natoms, size_t idx)
{
    const double *c = boxes + box_stride * idx;
    static const double zero3[3] = {0.0, 0.0, 0.0};
    double x0[3] = {c[3], c[4], c[5]};
    for (size_t a = 0; a < natoms; ++a) {
        double *xa = pos + idx * natoms * 3 + a * 3;
        for (int k = 0; k < 3; ++k) xa[k] = xa[k] - x0[k];
        oracle_min_image(xa, c + 3, tric ? c + 6 : zero3, tric);
        for (int k = 0; k < 3; ++k) xa[k] = xa[k] + x0[k];
    }
}

typedef struct {
    const double *pos;      /* [nframes][natoms][3], internal (post-preprocessing) */
    const double *boxes;    /* [nframes][box_stride], internal format */
    size_t box_stride;
    int tric;
    const int *type_ids;    /* [natoms], dense 0..ntypes-1 */
    unsigned ntypes;
    size_t natoms;
    double rmin, rmax;
    unsigned nbin;
    unsigned nch;
    size_t primo;
    /* per (lag, origin) */
    long t, imedia;
    size_t a0, a1;
    uint64_t *counts;       /* this thread's [leff][nch][nbin] */
} oracle_job;

/* One thread's share of one (lag, origin): gofrt.cpp:96-122. */
static void oracle_pairs(const oracle_job *j)
{
    size_t fo = j->primo + (size_t)j->imedia, fl = fo + (size_t)j->t;
    const double *box = j->boxes + fo * j->box_stride;
    unsigned half = j->ntypes * (j->ntypes + 1) / 2;
    for (size_t ia = j->a0; ia < j->a1; ++ia) {
        const double *xi = j->pos + (fo * j->natoms + ia) * 3;
        for (size_t ja = 0; ja < j->natoms; ++ja) {
            const double *xj = j->pos + (fl * j->natoms + ja) * 3;
            double d2 = oracle_d2(xi, xj, box, j->tric);
            int b = oracle_bin(d2, j->rmin, j->rmax, j->nbin);
            if (b < 0) continue;
            unsigned ch = oracle_channel((unsigned)j->type_ids[ia], (unsigned)j->type_ids[ja], j->ntypes);
            if (ia == ja) ch += half;
            j->counts[((size_t)j->t * j->nch + ch) * j->nbin + (unsigned)b] += 1;
        }
    }
}

static void *oracle_thread_main(void *arg)
{
    oracle_pairs((const oracle_job *)arg);
    return NULL;
}

/*
 * Integer counts of the Gofrt histogram, per thread partition.
 *
 * counts: [nthreads][leff][nch][nbin] u64, zeroed here.  Partition p holds the
 * pairs whose first atom lies in thread p's range of the reference's atom
 * split (calculatemultithread.h:50-78,87-89: [p*(N/nth), (p+1)*(N/nth)), the
 * last thread up to N), so that the reference's double buffer can be rebuilt
 * bit for bit (oracle_fold_buffer).  Threads are created and joined once per
 * (lag, origin), exactly as the reference's fork/join loop does
 * (calculatemultithread.h:114-151); this is also the timed CPU baseline.
 *
 * Returns 0, or -1 when leff+ntimesteps+primo > nframes+1 (the reference
 * throws, gofrt.cpp:81-83), or -2 on allocation failure.
 */
int oracle_gofrt_counts(const double *pos, const double *boxes, size_t box_stride, int tric,
                        const int *type_ids, unsigned ntypes, size_t natoms, size_t nframes,
                        double rmin, double rmax, unsigned nbin, unsigned tmax,
                        unsigned nthreads, unsigned skip, unsigned every,
                        unsigned ntimesteps, size_t primo, uint64_t *counts)
{
    if (nthreads == 0) nthreads = 1;
    if (skip == 0) skip = 1;
    if (every == 0) every = 1;
    unsigned leff = (ntimesteps < tmax || tmax == 0) ? ntimesteps : tmax;
    unsigned nch = ntypes * (ntypes + 1);
    size_t data_length = (size_t)leff * nch * nbin;
    memset(counts, 0, sizeof(uint64_t) * data_length * nthreads);
    if ((size_t)leff + ntimesteps + primo > nframes + 1) return -1;
    oracle_job *jobs = (oracle_job *)calloc(nthreads, sizeof(oracle_job));
    pthread_t *th = (pthread_t *)calloc(nthreads, sizeof(pthread_t));
    if (!jobs || !th) { free(jobs); free(th); return -2; }
    size_t per = natoms / nthreads;
    for (long t = 0; t < (long)leff; t += every) {
        for (long im = 0; im < (long)ntimesteps; im += skip) {
            for (unsigned p = 0; p < nthreads; ++p) {
                oracle_job *j = &jobs[p];
                j->pos = pos; j->boxes = boxes; j->box_stride = box_stride; j->tric = tric;
                j->type_ids = type_ids; j->ntypes = ntypes; j->natoms = natoms;
                j->rmin = rmin; j->rmax = rmax; j->nbin = nbin; j->nch = nch; j->primo = primo;
                j->t = t; j->imedia = im;
                j->a0 = p * per;
                j->a1 = (p == nthreads - 1) ? natoms : (p + 1) * per;
                j->counts = counts + data_length * p;
                if (nthreads == 1) oracle_pairs(j);
                else pthread_create(&th[p], NULL, oracle_thread_main, j);
            }
            if (nthreads > 1)
                for (unsigned p = 0; p < nthreads; ++p) pthread_join(th[p], NULL);
        }
    }
    free(jobs);
    free(th);
    return 0;
}

/* incr of the reference (gofrt.cpp:91-92): 1/int(ntimesteps/skip), or 1. */
double oracle_incr(unsigned ntimesteps, unsigned skip)
{
    if (skip == 0) skip = 1;
    if (ntimesteps / skip > 0) return 1.0 / (int)(ntimesteps / skip);
    return 1.0;
}

/*
 * The reference's double buffer rebuilt from per-partition counts:
 * each thread's bin is incr added k times in sequence (gofrt.cpp:118), and
 * thread buffers are folded into thread 0's in thread order (gofrt.cpp:128-132).
 */
void oracle_fold_buffer(const uint64_t *counts, size_t data_length, unsigned nthreads,
                        double incr, double *out)
{
    for (size_t i = 0; i < data_length; ++i) {
        double acc = 0.0;
        for (unsigned p = 0; p < nthreads; ++p) {
            double s = 0.0;
            for (uint64_t k = 0; k < counts[data_length * p + i]; ++k) s += incr;
            if (p == 0) acc = s; else acc += s;
        }
        out[i] = acc;
    }
}

/*
 * Per-frame, per-type centres of mass: running mean over the atoms of each
 * type, in atom order, of the given positions (Trajectory_numpy::calc_cm_pos_vel,
 * lib/src/trajectory_numpy.cpp:201-222).  cm: [T][ntypes][3].
 */
void oracle_centres(const double *pos, const int *type_ids, unsigned ntypes, size_t natoms,
                    size_t nframes, double *cm)
{
    unsigned *cont = (unsigned *)calloc(ntypes ? ntypes : 1, sizeof(unsigned));
    for (size_t f = 0; f < nframes; ++f) {
        for (unsigned k = 0; k < ntypes; ++k) {
            cont[k] = 0;
            for (int c = 0; c < 3; ++c) cm[(f * ntypes + k) * 3 + c] = 0.0;
        }
        for (size_t a = 0; a < natoms; ++a) {
            const unsigned k = (unsigned)type_ids[a];
            cont[k]++;
            for (int c = 0; c < 3; ++c) {
                double *m = &cm[(f * ntypes + k) * 3 + c];
                *m += (pos[(f * natoms + a) * 3 + c] - *m) / (double)cont[k];
            }
        }
    }
    free(cont);
}

/*
 * MSD<T>::calc_single_th for every lag (lib/src/msd.cpp:70-118): per lag t and
 * type, the running mean over origins imedia = 0, skip, ... < ntimesteps and
 * atoms (in that order) of pow(dx,2)+pow(dy,2)+pow(dz,2), dx = x(primo+imedia)
 * - x(primo+imedia+t) [- (cm(o) - cm(o+t)) with cm_self]; with cm_msd also the
 * running mean over origins of the centres' own squared displacement.  The
 * reference splits lags over threads (PARALLEL_SPLIT_TIME); each lag's value
 * does not depend on that split.  out: [leff][f_cm][ntypes].  Returns -1 when
 * leff + ntimesteps + primo > nframes (msd.cpp:57-60).
 */
int oracle_msd(const double *pos, const double *cm, const int *type_ids, unsigned ntypes,
               size_t natoms, size_t nframes, unsigned skip, unsigned tmax, unsigned ntimesteps,
               size_t primo, int cm_msd, int cm_self, double *out)
{
    const size_t leff = (ntimesteps < tmax || tmax == 0) ? ntimesteps : tmax;
    const size_t f_cm = cm_msd ? 2 : 1;
    if (skip == 0) skip = 1;
    if (leff + ntimesteps + primo > nframes) return -1;
    uint64_t *cont = (uint64_t *)calloc(ntypes * f_cm + 1, sizeof(uint64_t));
    for (size_t t = 0; t < leff; ++t) {
        double *v = out + t * ntypes * f_cm;
        for (size_t i = 0; i < ntypes * f_cm; ++i) {
            v[i] = 0.0;
            cont[i] = 0;
        }
        for (size_t im = 0; im < ntimesteps; im += skip) {
            const size_t fo = primo + im, fl = primo + im + t;
            for (size_t a = 0; a < natoms; ++a) {
                const unsigned k = (unsigned)type_ids[a];
                const double *xo = pos + (fo * natoms + a) * 3;
                const double *xl = pos + (fl * natoms + a) * 3;
                double d[3];
                for (int c = 0; c < 3; ++c) {
                    d[c] = xo[c] - xl[c];
                    if (cm_self)
                        d[c] = d[c] - (cm[(fo * ntypes + k) * 3 + c] - cm[(fl * ntypes + k) * 3 + c]);
                }
                const double delta = (pow(d[0], 2) + pow(d[1], 2) + pow(d[2], 2)) - v[k];
                v[k] += delta / (double)(++cont[k]);
            }
            if (cm_msd) {
                for (unsigned k = 0; k < ntypes; ++k) {
                    const double *co = cm + (fo * ntypes + k) * 3;
                    const double *cl = cm + (fl * ntypes + k) * 3;
                    const double delta = (pow(co[0] - cl[0], 2) + pow(co[1] - cl[1], 2) +
                                          pow(co[2] - cl[2], 2)) - v[ntypes + k];
                    v[ntypes + k] += delta / (double)(++cont[ntypes + k]);
                }
            }
        }
    }
    free(cont);
    return 0;
}

/*
 * Neighbours<T,double>::update_neigh (lib/src/neighbour.cpp:9-79), literally:
 * for i < j (i outer), d2 and x = x_i - x_j by the minimum image of frame
 * `timestep`; a pair within either type's cutoff goes into i's list of j's
 * type and j's list of i's type (written at the current size, counted only
 * within the cutoff of the neighbour's type); a full list when such a pair
 * arrives is the reference's "Too many neighbours in shell!" (returns -1 and
 * err_info = {iatom, jatom, ni, nj, itype, jtype}).  Optional sort of every
 * list by distance: a stable insertion sort (what std::sort does for up to 16
 * elements; with ties in longer lists the reference's order is unspecified).
 * Layout (neighbour.h:68-96): list[list_off[k] + i (nneigh[k]+1)] = size, then
 * the indices; rpos[rpos_off[k] + i nneigh[k] 4 + 4 n] = {r, x, y, z}.
 */
int oracle_neigh(const double *pos, const double *boxes, size_t box_stride, int tric,
                 const int *type_ids, unsigned ntypes, size_t natoms, size_t timestep,
                 const uint64_t *nneigh, const double *cut2, int sort, uint64_t *list,
                 double *rpos, uint64_t *err_info)
{
    size_t *loff = (size_t *)calloc(ntypes + 1, sizeof(size_t));
    size_t *roff = (size_t *)calloc(ntypes + 1, sizeof(size_t));
    size_t total = 0, max_n = 0;
    for (unsigned k = 0; k < ntypes; ++k) {
        loff[k + 1] = loff[k] + (nneigh[k] + 1) * natoms;
        roff[k + 1] = roff[k] + nneigh[k] * natoms * 4;
        total += nneigh[k];
        if (nneigh[k] > max_n) max_n = nneigh[k];
    }
    for (size_t i = 0; i < natoms * (total + ntypes); ++i) list[i] = 0;
    const double *box = boxes + timestep * box_stride;
    static const double zero3[3] = {0.0, 0.0, 0.0};
    int rc = 0;
    for (size_t i = 0; i < natoms && rc == 0; ++i) {
        const unsigned it = (unsigned)type_ids[i];
        for (size_t j = i + 1; j < natoms; ++j) {
            const unsigned jt = (unsigned)type_ids[j];
            const double *xi = pos + (timestep * natoms + i) * 3;
            const double *xj = pos + (timestep * natoms + j) * 3;
            double x[3], d2 = 0.0;
            for (int c = 0; c < 3; ++c) x[c] = xi[c] - xj[c];
            oracle_min_image(x, box + 3, tric ? box + 6 : zero3, tric);
            for (int c = 0; c < 3; ++c) d2 += x[c] * x[c];
            if (d2 <= cut2[jt] || d2 <= cut2[it]) {
                uint64_t *il = list + loff[jt] + i * (nneigh[jt] + 1);
                uint64_t *jl = list + loff[it] + j * (nneigh[it] + 1);
                const uint64_t ni = il[0], nj = jl[0];
                if (ni < nneigh[jt] && nj < nneigh[it]) {
                    const double r = sqrt(d2);
                    il[1 + ni] = j;
                    jl[1 + nj] = i;
                    double *ip = rpos + roff[jt] + i * nneigh[jt] * 4 + ni * 4;
                    double *jp = rpos + roff[it] + j * nneigh[it] * 4 + nj * 4;
                    ip[0] = r;
                    jp[0] = r;
                    for (int c = 0; c < 3; ++c) {
                        ip[1 + c] = x[c];
                        jp[1 + c] = -x[c];
                    }
                    if (d2 <= cut2[jt]) il[0]++;
                    if (d2 <= cut2[it]) jl[0]++;
                } else {
                    err_info[0] = i; err_info[1] = j; err_info[2] = ni; err_info[3] = nj;
                    err_info[4] = it; err_info[5] = jt;
                    rc = -1;
                    break;
                }
            }
        }
    }
    if (rc == 0 && sort) {
        for (unsigned k = 0; k < ntypes; ++k) {
            for (size_t a = 0; a < natoms; ++a) {
                uint64_t *l = list + loff[k] + a * (nneigh[k] + 1);
                double *rp = rpos + roff[k] + a * nneigh[k] * 4;
                const size_t n = l[0];
                for (size_t s = 1; s < n; ++s) {
                    double e[4];
                    memcpy(e, rp + 4 * s, sizeof e);
                    const uint64_t id = l[1 + s];
                    size_t q = s;
                    while (q > 0 && e[0] < rp[4 * (q - 1)]) {
                        memcpy(rp + 4 * q, rp + 4 * (q - 1), sizeof e);
                        l[1 + q] = l[q];
                        --q;
                    }
                    memcpy(rp + 4 * q, e, sizeof e);
                    l[1 + q] = id;
                }
            }
        }
    }
    (void)max_n;
    free(loff);
    free(roff);
    return rc;
}

/* Neighbours::get_sann_n (lib/src/neighbour.cpp:82-97) on one list's
 * distances r[0..n) (sorted). */
uint64_t oracle_sann_n(const double *rpos4, uint64_t n)
{
    if (n < 3) return 0;
    uint64_t m = 3;
    double s = 0.0;
    for (uint64_t i = 0; i < m; ++i) s += rpos4[4 * i];
    while (m < n) {
        if (s <= rpos4[4 * m] * (m - 2)) break;
        s += rpos4[4 * m];
        m++;
    }
    return m;
}
