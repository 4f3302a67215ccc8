// Block averages of a calculation over a trajectory: the driver the CLI's
// g(r,t) branch uses (lib/include/blockaverage.h:107-190 with MediaVar,
// lib/include/calcoliblocchi.h:21-61).
//
// The trajectory is split into n_b blocks of s = (T - nExtraTimesteps(n_b))/n_b
// origins-window each; block i runs calculate(i*s) on the resident frames and
// feeds an online mean/variance.  The reference re-reads and re-wraps a window
// of the memory-mapped file for every block; here every frame is already in
// HBM, so a block is one engine launch.
#pragma once
#include <cstdlib>
#include <iostream>
#include <memory>
#include <stdexcept>

namespace analisi_gb300 {

// Online mean and variance (lib/include/calcoliblocchi.h:21-61), elementwise
// on the calculation objects with the reference's operation order.
template <class T>
class MediaVar {
public:
    MediaVar(T *mean, T *var, T *delta, T *tmp) : Tmedio(mean), Tvar(var), delta(delta), tmp(tmp) {}
    void calcola_begin(unsigned s)
    {
        Tmedio->reset(s);
        Tmedio->azzera();
        Tvar->reset(s);
        Tvar->azzera();
        delta->reset(s);
        tmp->reset(s);
        iblock = 0;
    }
    void calculate(T *calcolo)
    {
        *delta = *calcolo;
        *delta -= *Tmedio;
        *tmp = *delta;
        *tmp /= (iblock + 1);
        *Tmedio += *tmp;
        *tmp = *calcolo;
        *tmp -= *Tmedio;
        *tmp *= *delta;
        *Tvar += *tmp;
        iblock++;
    }
    void calcola_end(unsigned n_b) { *Tvar /= ((n_b - 1) * n_b); }

private:
    T *Tmedio, *Tvar, *delta, *tmp;
    unsigned iblock = 0;
};

template <class TR, class T>
class BlockAverage {
public:
    BlockAverage(TR *t, unsigned n_blocks) : traj(t), n_b(n_blocks) {}

    template <typename... Args>
    void calculate(Args... args)
    {
        Tmedio.reset(new T(traj, args...));
        Tvar.reset(new T(traj, args...));
        delta.reset(new T(traj, args...));
        tmp.reset(new T(traj, args...));
        calcolo.reset(new T(traj, args...));
        MediaVar<T> mv(Tmedio.get(), Tvar.get(), delta.get(), tmp.get());
        const long long per =
            ((long long)traj->get_ntimesteps() - (long long)calcolo->nExtraTimesteps(n_b)) / n_b;
        if (per <= 0) {
            std::cerr << "Cannot divide the trajectory in " << n_b << " blocks!\n";
            std::abort();
        }
        s = (unsigned)per;
        calcolo->reset(s);
        mv.calcola_begin(s);
        for (unsigned iblock = 0; iblock < n_b; iblock++) {
            calcolo->reset(s);
            calcolo->calculate((size_t)iblock * s);
            mv.calculate(calcolo.get());
        }
        mv.calcola_end(n_b);
        ok = true;
    }

    T *media() { return checked(Tmedio.get()); }
    T *varianza() { return checked(Tvar.get()); }
    T *puntatoreCalcolo() { return checked(calcolo.get()); }
    unsigned block_size() const { return s; }

private:
    T *checked(T *p)
    {
        if (!ok) std::abort();
        return p;
    }
    TR *traj;
    unsigned n_b, s = 0;
    bool ok = false;
    std::unique_ptr<T> Tmedio, Tvar, delta, tmp, calcolo;
};

}  // namespace analisi_gb300
