// Gofrt<TFLOAT, T>: the reference's g(r,t) calculation object
// (lib/include/gofrt.h:28-107, lib/src/gofrt.cpp), same constructor, members
// and result buffer, with the calculation done by the GB300 engine behind the
// C ABI of include/gofr_gb300.h.
//
// T is a trajectory providing the reference's internal buffers:
// get_natoms(), get_ntimesteps(), get_ntypes(), positions_data(), box(0)
// (all frames' boxes, get_box_stride() doubles each), is_triclinic(),
// type_ids() (dense ids) and data_version() (changes when the buffers change;
// the frames are re-uploaded then).  analisi_gb300::Trajectory is one.
//
// The result buffer (access_vdata(), shape (leff, ntypes(ntypes+1), nbin),
// byte strides as lib/src/gofrt.cpp:65-71) holds exactly the reference's
// doubles: counts are computed per reference thread partition (nthreads) and
// folded as the reference's threads would have added incr.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <sys/types.h>
#include <type_traits>
#include <utility>
#include <vector>

#include "gofr_gb300.h"

namespace analisi_gb300 {

// Trajectories that hold a window of their frames (TrajWindow: window_start,
// window_frames, ensure_window) rather than all of them.
template <class T, class = void>
struct has_window : std::false_type {};
template <class T>
struct has_window<T, std::void_t<decltype(std::declval<T &>().window_start())>>
    : std::true_type {};

template <class TFLOAT, class T>
class Gofrt {
public:
    Gofrt(T *t, TFLOAT rmin, TFLOAT rmax, unsigned int nbin, unsigned int tmax = 0,
          unsigned int nthreads = 0, unsigned int skip = 1, unsigned int every = 1,
          bool debug = false)
        : traiettoria(t), rmin(rmin), rmax(rmax), nbin(nbin), lmax(tmax),
          nthreads(nthreads ? nthreads : 1), skip(skip ? skip : 1), every(every ? every : 1),
          debug(debug)
    {
        // the reference normalises 0 to 1 for threads, skip and every
        // (lib/include/calculatemultithread.h:41-47)
        if (const char *k = std::getenv("ANALISI_GB300_KERNEL")) kernel = std::atoi(k);
        if (const char *d = std::getenv("ANALISI_GB300_DEVICE")) device = std::atoi(d);
        // frames beyond this many device bytes are streamed through the GPU in
        // chunks of origins instead of being held resident (0: no limit)
        if (const char *b = std::getenv("ANALISI_GB300_DEVICE_BUDGET"))
            device_budget = (size_t)std::strtod(b, nullptr);
    }
    ~Gofrt()
    {
        if (ctx) gofr_ctx_destroy(ctx);
    }
    Gofrt(const Gofrt &o) : Gofrt(o.traiettoria, o.rmin, o.rmax, o.nbin, o.lmax, o.nthreads,
                                  o.skip, o.every, o.debug)
    {
        leff = o.leff;
        ntimesteps = o.ntimesteps;
        vdata = o.vdata;
        c_descr = o.c_descr;
    }

    // lib/src/gofrt.cpp:41-63
    void reset(const unsigned int numeroTimestepsPerBlocco)
    {
        std::stringstream descr;
        const unsigned nt = ntypes();
        descr << "# The first column is the time difference in timesteps, then you have the bin "
                 "index. Every column after is followed by the variance. Then you have the "
                 "following: " << std::endl;
        for (unsigned t1 = 0; t1 < nt; t1++) {
            for (unsigned t2 = t1; t2 < nt; t2++) {
                descr << "#g(" << t1 << ", " << t2 << "), different atom index: "
                      << get_itype(t1, t2) * 2 + 3 << std::endl;
                descr << "#g(" << t1 << ", " << t2 << "), same atom index: "
                      << (get_itype(t1, t2) + nt * (nt + 1) / 2) * 2 + 3 << std::endl;
            }
        }
        descr << "# same atom index means that the atom is tracked around and the average "
                 "self-spread is shown with larger time differences." << std::endl;
        descr << "# different atom index is something that for t=0 is the traditional g(r) "
              << std::endl;
        c_descr = descr.str();
        leff = (numeroTimestepsPerBlocco < lmax || lmax == 0) ? numeroTimestepsPerBlocco : lmax;
        ntimesteps = numeroTimestepsPerBlocco;
        vdata.assign((size_t)leff * nt * (nt + 1) * nbin, TFLOAT(0));
    }

    // lib/src/gofrt.cpp:37-39
    unsigned int nExtraTimesteps(unsigned int n_b)
    {
        const size_t nts = traiettoria->get_ntimesteps();
        return (nts / (n_b + 1) + 1 < lmax || lmax == 0) ? nts / (n_b + 1) + 1 : lmax;
    }

    // CalculateMultiThread::calculate + calc_init/calc_single_th/calc_end
    // (lib/include/calculatemultithread.h:106-162, lib/src/gofrt.cpp:74-155)
    void calculate(size_t primo)
    {
        size_t rel = primo;
        if constexpr (has_window<T>::value) {
            // the frames of every origin and lag: [primo, primo + n + leff - 1)
            const size_t need = ntimesteps + leff > 1 ? ntimesteps + leff - 1 : 1;
            traiettoria->ensure_window(primo, need);
            rel = primo - traiettoria->window_start();
        }
        const size_t nframes = frames();
        const bool stream = device_budget > 0 &&
                            (double)nframes * traiettoria->get_natoms() * 64.0 > (double)device_budget;
        if (stream) make_ctx();
        else ensure_frames();
        gofr_params p{};
        p.rmin = rmin;
        p.rmax = rmax;
        p.nbin = nbin;
        p.tmax = lmax;
        p.skip = skip;
        p.every = every;
        p.ntimesteps = ntimesteps;
        p.primo = rel;
        p.kernel = kernel;
        p.nparts = nthreads;
        size_t n = 0;
        if (stream) {
            const unsigned nt = ntypes();
            n = (size_t)leff * nt * (nt + 1) * nbin * (nthreads > 1 ? nthreads : 1);
            counts.resize(n ? n : 1);
            check(gofr_run_streamed(ctx, traiettoria->positions_data(), traiettoria->box(0),
                                    traiettoria->is_triclinic() ? GOFR_BOX_TRICLINIC
                                                                : GOFR_BOX_ORTHO,
                                    traiettoria->type_ids(), nt, traiettoria->get_natoms(),
                                    nframes, &p, device_budget, counts.data()));
            uploaded_version = ~0ull;  // the context holds the last chunk's frames
        } else {
            check(gofr_output_size(ctx, &p, &n));
            counts.resize(n ? n : 1);
            check(gofr_run(ctx, &p, counts.data()));
        }
        const size_t dl = vdata.size();
        if (n == 0 || dl == 0) return;
        std::vector<double> tmp;
        double *dst = nullptr;
        if constexpr (sizeof(TFLOAT) == sizeof(double)) dst = reinterpret_cast<double *>(vdata.data());
        else { tmp.resize(dl); dst = tmp.data(); }
        check(gofr_counts_to_buffer(counts.data(), dl, nthreads, ntimesteps, skip, dst));
        if constexpr (sizeof(TFLOAT) != sizeof(double))
            for (size_t i = 0; i < dl; ++i) vdata[i] = (TFLOAT)tmp[i];
        if (debug) dump();
    }

    std::vector<ssize_t> get_shape()
    {
        const unsigned nt = ntypes();
        return {(ssize_t)leff, (ssize_t)(nt * (nt + 1)), (ssize_t)nbin};
    }
    std::vector<ssize_t> get_stride()
    {
        const unsigned nt = ntypes();
        return {(ssize_t)(nt * (nt + 1) * nbin * sizeof(TFLOAT)), (ssize_t)(nbin * sizeof(TFLOAT)),
                (ssize_t)sizeof(TFLOAT)};
    }
    std::string get_columns_description() { return c_descr; }

    // VectorOp members used by the buffer protocol and the block averages
    // (lib/include/operazionisulista.h:25-148)
    TFLOAT *access_vdata() { return vdata.data(); }
    unsigned int lunghezza() const { return (unsigned)vdata.size(); }
    TFLOAT elemento(unsigned int i) const
    {
        if (i < vdata.size()) return vdata[i];
        throw std::runtime_error("Out of range index");
    }
    void azzera()
    {
        for (auto &v : vdata) v = 0;
    }
    Gofrt &operator=(const Gofrt &o)
    {
        vdata = o.vdata;  // reallocates when the length differs, as VectorOp::operator=
        return *this;
    }
    Gofrt &operator+=(const Gofrt &o) { return elementwise(o, [](TFLOAT &a, TFLOAT b) { a += b; }); }
    Gofrt &operator-=(const Gofrt &o) { return elementwise(o, [](TFLOAT &a, TFLOAT b) { a -= b; }); }
    Gofrt &operator*=(const Gofrt &o) { return elementwise(o, [](TFLOAT &a, TFLOAT b) { a *= b; }); }
    Gofrt &operator/=(const Gofrt &o) { return elementwise(o, [](TFLOAT &a, TFLOAT b) { a /= b; }); }
    Gofrt &operator+=(const TFLOAT &s) { for (auto &v : vdata) v += s; return *this; }
    Gofrt &operator-=(const TFLOAT &s) { for (auto &v : vdata) v -= s; return *this; }
    Gofrt &operator*=(const TFLOAT &s) { for (auto &v : vdata) v *= s; return *this; }
    Gofrt &operator/=(const TFLOAT &s) { for (auto &v : vdata) v /= s; return *this; }

    // engine statistics of the last calculate (pairs, rechecks, device time)
    gofr_stats last_stats() const
    {
        gofr_stats s{};
        if (ctx) gofr_get_stats(ctx, &s);
        return s;
    }
    void set_kernel(int k) { kernel = k; }
    void set_device_budget(size_t bytes) { device_budget = bytes; }

private:
    unsigned ntypes() const { return (unsigned)traiettoria->get_ntypes(); }

    // lib/include/gofrt.h:86-104
    unsigned get_itype(unsigned type1, unsigned type2) const
    {
        if (type2 < type1) std::swap(type1, type2);
        const unsigned nt = ntypes();
        return nt * (nt + 1) / 2 - (type2 + 1) * (type2 + 2) / 2 + type1;
    }

    template <class F>
    Gofrt &elementwise(const Gofrt &o, F f)
    {
        if (o.lunghezza() != lunghezza())
            throw std::runtime_error("Trying to operate on VectorOp of different sizes!");
        for (size_t i = 0; i < vdata.size(); ++i) f(vdata[i], o.vdata[i]);
        return *this;
    }

    void check(int rc)
    {
        if (rc != GOFR_OK) throw std::runtime_error(gofr_last_error(ctx));
    }

    // frames held by the trajectory: its window, or all of them
    size_t frames() const
    {
        if constexpr (has_window<T>::value) return traiettoria->window_frames();
        else return traiettoria->get_ntimesteps();
    }

    void make_ctx()
    {
        if (!ctx) {
            if (gofr_ctx_create(&ctx, device) != GOFR_OK)
                throw std::runtime_error(std::string("gofr: cannot create a GPU context: ") +
                                         gofr_last_error(nullptr));
        }
    }

    void ensure_frames()
    {
        make_ctx();
        const auto ver = traiettoria->data_version();
        if (uploaded_version != ver) {
            check(gofr_set_frames(ctx, traiettoria->positions_data(), traiettoria->box(0),
                                  traiettoria->is_triclinic() ? GOFR_BOX_TRICLINIC
                                                              : GOFR_BOX_ORTHO,
                                  traiettoria->type_ids(), ntypes(), traiettoria->get_natoms(),
                                  frames()));
            uploaded_version = ver;
        }
    }

    // lib/src/gofrt.cpp:137-153
    void dump()
    {
        std::ofstream out("gofrt.dump", std::ios::app);
        const unsigned nch = ntypes() * (ntypes() + 1);
        for (unsigned ts = 0; ts < leff; ts++) {
            for (unsigned r = 0; r < nbin; r++) {
                out << ts << " " << r;
                for (unsigned itype = 0; itype < nch; itype++)
                    out << " " << vdata[(size_t)ts * nch * nbin + (size_t)nbin * itype + r];
                out << "\n";
            }
        }
        out << "\n\n";
    }

    T *traiettoria;
    TFLOAT rmin, rmax;
    unsigned int nbin, lmax, nthreads, skip, every;
    bool debug;
    unsigned int leff = 0, ntimesteps = 0;
    std::vector<TFLOAT> vdata;
    std::vector<unsigned long long> counts;
    std::string c_descr;
    gofr_ctx *ctx = nullptr;
    int device = 0;
    int kernel = GOFR_KERNEL_AUTO;
    size_t device_budget = 0;
    unsigned long long uploaded_version = ~0ull;
};

}  // namespace analisi_gb300
