// MeanSquareDisplacement<T>: the reference's MSD<T> (lib/include/msd.h:25-58,
// lib/src/msd.cpp:24-148), same constructor, members and result buffer, with
// the calculation done on the GPU behind the C ABI of include/gofr_gb300.h
// (gofr_msd_run on the trajectory's resident frames).
//
// T is a trajectory providing the reference's internal buffers (see
// gofrt.h) plus centres_data(), the per-frame per-type centres of mass
// [T][ntypes][3] of the reference's positions_cm.  analisi_gb300::Trajectory
// is one.
//
// The result buffer (access_vdata(), shape (leff, f_cm, ntypes), byte strides
// as lib/include/msd.h:37-38) holds, per lag and type, the mean over origins
// and atoms of the squared displacement; the reference keeps a running mean,
// the GPU sums in a fixed order and divides, so the two agree to rounding.
#pragma once
#include <cstdlib>
#include <fstream>
#include <stdexcept>
#include <string>
#include <sys/types.h>
#include <vector>

#include "gofr_gb300.h"

namespace analisi_gb300 {

template <class T>
class MeanSquareDisplacement {
public:
    MeanSquareDisplacement(T *t, unsigned int skip = 1, unsigned int tmax = 0,
                           unsigned int nthreads = 0, bool calcola_msd_centro_di_massa = false,
                           bool calcola_msd_nel_sistema_del_centro_di_massa = false,
                           bool debug = false)
        : traiettoria(t), lmax(tmax), skip(skip ? skip : 1), nthreads(nthreads),
          cm_msd(calcola_msd_centro_di_massa),
          cm_self(calcola_msd_nel_sistema_del_centro_di_massa), debug(debug),
          f_cm(calcola_msd_centro_di_massa ? 2 : 1)
    {
        if (const char *d = std::getenv("ANALISI_GB300_DEVICE")) device = std::atoi(d);
    }
    ~MeanSquareDisplacement()
    {
        if (ctx) gofr_ctx_destroy(ctx);
    }
    MeanSquareDisplacement(const MeanSquareDisplacement &o)
        : MeanSquareDisplacement(o.traiettoria, o.skip, o.lmax, o.nthreads, o.cm_msd, o.cm_self,
                                 o.debug)
    {
        leff = o.leff;
        ntimesteps = o.ntimesteps;
        ntypes = o.ntypes;
        vdata = o.vdata;
    }

    // lib/src/msd.cpp:37-39
    unsigned int nExtraTimesteps(unsigned int n_b)
    {
        const size_t nts = traiettoria->get_ntimesteps();
        return (nts / (n_b + 1) + 1 < lmax || lmax == 0) ? nts / (n_b + 1) + 1 : lmax;
    }

    // lib/src/msd.cpp:41-52
    void reset(const unsigned int numeroTimestepsPerBlocco)
    {
        leff = (numeroTimestepsPerBlocco < lmax || lmax == 0) ? numeroTimestepsPerBlocco : lmax;
        ntypes = traiettoria->get_ntypes();
        ntimesteps = numeroTimestepsPerBlocco;
        vdata.assign((size_t)leff * ntypes * f_cm, 0.0);
    }

    // CalculateMultiThread::calculate + calc_init/calc_single_th/calc_end
    // (lib/src/msd.cpp:54-139)
    void calculate(size_t primo)
    {
        ensure_frames();
        gofr_msd_params p{};
        p.skip = skip;
        p.tmax = lmax;
        p.ntimesteps = ntimesteps;
        p.primo = primo;
        p.center_of_mass = cm_msd ? 1 : 0;
        p.in_center_of_mass_frame = cm_self ? 1 : 0;
        size_t n = 0;
        check(gofr_msd_output_size(ctx, &p, &n));
        if (n != vdata.size()) vdata.assign(n, 0.0);
        if (n == 0) {
            // the reference still checks the trajectory length (msd.cpp:57-60)
            std::vector<double> one(1);
            check(gofr_msd_run(ctx, &p, one.data()));
        } else {
            check(gofr_msd_run(ctx, &p, vdata.data()));
        }
        if (debug) dump();
    }

    std::vector<ssize_t> get_shape() const
    {
        return {(ssize_t)leff, (ssize_t)f_cm, (ssize_t)ntypes};
    }
    std::vector<ssize_t> get_stride() const
    {
        return {(ssize_t)(ntypes * f_cm * sizeof(double)), (ssize_t)(ntypes * sizeof(double)),
                (ssize_t)sizeof(double)};
    }

    // VectorOp members (lib/include/operazionisulista.h:25-148)
    double *access_vdata() { return vdata.data(); }
    unsigned int lunghezza() const { return (unsigned)vdata.size(); }
    double elemento(unsigned int i) const
    {
        if (i < vdata.size()) return vdata[i];
        throw std::runtime_error("Out of range index");
    }
    void azzera()
    {
        for (auto &v : vdata) v = 0;
    }
    MeanSquareDisplacement &operator=(const MeanSquareDisplacement &o)
    {
        vdata = o.vdata;
        return *this;
    }
    MeanSquareDisplacement &operator+=(const MeanSquareDisplacement &o)
    {
        return elementwise(o, [](double &a, double b) { a += b; });
    }
    MeanSquareDisplacement &operator-=(const MeanSquareDisplacement &o)
    {
        return elementwise(o, [](double &a, double b) { a -= b; });
    }
    MeanSquareDisplacement &operator*=(const MeanSquareDisplacement &o)
    {
        return elementwise(o, [](double &a, double b) { a *= b; });
    }
    MeanSquareDisplacement &operator/=(const MeanSquareDisplacement &o)
    {
        return elementwise(o, [](double &a, double b) { a /= b; });
    }
    MeanSquareDisplacement &operator*=(const double &s)
    {
        for (auto &v : vdata) v *= s;
        return *this;
    }
    MeanSquareDisplacement &operator/=(const double &s)
    {
        for (auto &v : vdata) v /= s;
        return *this;
    }

    gofr_stats last_stats() const
    {
        gofr_stats s{};
        if (ctx) gofr_get_stats(ctx, &s);
        return s;
    }

private:
    template <class F>
    MeanSquareDisplacement &elementwise(const MeanSquareDisplacement &o, F f)
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

    void ensure_frames()
    {
        if (!ctx) {
            if (gofr_ctx_create(&ctx, device) != GOFR_OK)
                throw std::runtime_error(std::string("gofr: cannot create a GPU context: ") +
                                         gofr_last_error(nullptr));
        }
        const auto ver = traiettoria->data_version();
        if (uploaded_version != ver) {
            check(gofr_set_frames(ctx, traiettoria->positions_data(), traiettoria->box(0),
                                  traiettoria->is_triclinic() ? GOFR_BOX_TRICLINIC
                                                              : GOFR_BOX_ORTHO,
                                  traiettoria->type_ids(), (unsigned)traiettoria->get_ntypes(),
                                  traiettoria->get_natoms(), traiettoria->get_ntimesteps()));
            check(gofr_set_centres(ctx, traiettoria->centres_data(),
                                   traiettoria->get_ntimesteps(),
                                   (unsigned)traiettoria->get_ntypes()));
            uploaded_version = ver;
        }
    }

    // lib/src/msd.cpp:121-139
    void dump()
    {
        std::ofstream out("msd.dump", std::ios::app);
        for (size_t ts = 0; ts < leff; ts++) {
            out << ts;
            for (size_t itype = 0; itype < ntypes * f_cm; itype++)
                out << " " << vdata[ntypes * ts * f_cm + itype];
            out << "\n";
        }
        out << "\n\n";
    }

    T *traiettoria;
    unsigned int lmax, skip, nthreads;
    bool cm_msd, cm_self, debug;
    size_t f_cm;
    size_t leff = 0, ntimesteps = 0, ntypes = 0;
    std::vector<double> vdata;
    gofr_ctx *ctx = nullptr;
    int device = 0;
    unsigned long long uploaded_version = ~0ull;
};

}  // namespace analisi_gb300
