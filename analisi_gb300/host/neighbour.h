// Neighbours<T, TType>: the reference's neighbour lists
// (lib/include/neighbour.h:9-104, lib/src/neighbour.cpp:9-97), same
// constructor, list layout and accessors, with update_neigh done on the GPU
// behind the C ABI of include/gofr_gb300.h (gofr_neigh_run on the
// trajectory's resident frames).  Only TType = double, as the reference
// instantiates it.
#pragma once
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "gofr_gb300.h"

namespace analisi_gb300 {

template <class T, class TType = double>
class Neighbours {
    static_assert(sizeof(TType) == sizeof(double), "the GPU lists are double");

public:
    using ListSpec = std::vector<std::tuple<size_t, TType, TType>>;
    using TType4 = TType[4];

    template <class TN>
    class NeighIterator {
    public:
        NeighIterator(TN *idxs, const size_t len) : idxs_(idxs), len_(len) {}
        const TN *begin() { return idxs_; }
        TN *begin_w() { return idxs_; }
        const TN *end() { return idxs_ + len_; }
        size_t size() const { return len_; }

    private:
        TN *idxs_;
        size_t len_;
    };

    // lib/include/neighbour.h:31-46
    Neighbours(T *t, const ListSpec nneigh_cut2_skin2) : t(*t), spec(nneigh_cut2_skin2)
    {
        if (t->get_ntypes() != spec.size())
            throw std::runtime_error(
                "In neighbours list you must specify parameters for each atomic type");
        size_t lo = 0, ro = 0;
        for (const auto &s : spec) {
            list_offset.push_back(lo);
            rpos_offset.push_back(ro);
            lo += (std::get<0>(s) + 1) * t->get_natoms();
            ro += std::get<0>(s) * t->get_natoms() * 4;
        }
        list.assign(lo, 0);
        rpos.assign(ro, 0.0);
        if (const char *d = std::getenv("ANALISI_GB300_DEVICE")) device = std::atoi(d);
    }
    ~Neighbours()
    {
        if (ctx) gofr_ctx_destroy(ctx);
    }
    Neighbours(const Neighbours &) = delete;
    Neighbours &operator=(const Neighbours &) = delete;

    // lib/src/neighbour.cpp:9-79
    void update_neigh(const size_t timestep, bool sort)
    {
        ensure_frames();
        std::vector<gofr_neigh_spec> s(spec.size());
        for (size_t k = 0; k < spec.size(); ++k)
            s[k] = {(unsigned long long)std::get<0>(spec[k]), (double)std::get<1>(spec[k]),
                    (double)std::get<2>(spec[k])};
        size_t nl = 0, nr = 0;
        check(gofr_neigh_layout(ctx, s.data(), (unsigned)s.size(), &nl, &nr));
        list.resize(nl);
        rpos.resize(nr);
        check(gofr_neigh_run(ctx, s.data(), (unsigned)s.size(), timestep, sort ? 1 : 0,
                             reinterpret_cast<unsigned long long *>(list.data()),
                             reinterpret_cast<double *>(rpos.data())));
    }

    // lib/include/neighbour.h:49-64
    NeighIterator<size_t> get_neigh(const size_t iatom, const size_t jtype)
    {
        size_t *b = list.data() + list_offset[jtype] + iatom * (nneigh(jtype) + 1);
        return NeighIterator<size_t>{b + 1, b[0]};
    }
    NeighIterator<TType4> get_neigh_r(const size_t iatom, const size_t jtype)
    {
        return NeighIterator<TType4>{
            reinterpret_cast<TType4 *>(rpos.data() + rpos_offset[jtype] +
                                       iatom * nneigh(jtype) * 4),
            list[list_offset[jtype] + iatom * (nneigh(jtype) + 1)]};
    }
    // lib/src/neighbour.cpp:82-97
    size_t get_sann_n(const size_t iatom, const size_t jtype)
    {
        auto r = get_neigh_r(iatom, jtype);
        if (r.size() < 3) return 0;
        size_t sann_n = 3;
        TType s = 0.0;
        for (size_t i = 0; i < sann_n; ++i) s += r.begin()[i][0];
        while (sann_n < r.size()) {
            if (s <= r.begin()[sann_n][0] * (sann_n - 2)) break;
            s += r.begin()[sann_n][0];
            sann_n++;
        }
        return sann_n;
    }
    NeighIterator<size_t> get_sann(const size_t iatom, const size_t jtype)
    {
        size_t *b = list.data() + list_offset[jtype] + iatom * (nneigh(jtype) + 1);
        return NeighIterator<size_t>{b + 1, get_sann_n(iatom, jtype)};
    }
    NeighIterator<TType4> get_sann_r(const size_t iatom, const size_t jtype)
    {
        return NeighIterator<TType4>{
            reinterpret_cast<TType4 *>(rpos.data() + rpos_offset[jtype] +
                                       iatom * nneigh(jtype) * 4),
            get_sann_n(iatom, jtype)};
    }

private:
    size_t nneigh(size_t itype) const { return std::get<0>(spec[itype]); }

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
        const auto ver = t.data_version();
        if (uploaded_version != ver) {
            check(gofr_set_frames(ctx, t.positions_data(), t.box(0),
                                  t.is_triclinic() ? GOFR_BOX_TRICLINIC : GOFR_BOX_ORTHO,
                                  t.type_ids(), (unsigned)t.get_ntypes(), t.get_natoms(),
                                  t.get_ntimesteps()));
            uploaded_version = ver;
        }
    }

    T &t;
    const ListSpec spec;
    std::vector<size_t> list_offset, rpos_offset;
    std::vector<size_t> list;
    std::vector<TType> rpos;
    gofr_ctx *ctx = nullptr;
    int device = 0;
    unsigned long long uploaded_version = ~0ull;
};

}  // namespace analisi_gb300
