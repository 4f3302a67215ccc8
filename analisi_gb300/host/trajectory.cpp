// Host-side trajectory preprocessing; see trajectory.h for what it restates.
#include "trajectory.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>

namespace analisi_gb300 {

// lammps {xlo,xhi,ylo,yhi,zlo,zhi} -> internal {xlo,ylo,zlo,lx/2,ly/2,lz/2}
// in place (lib/include/basetrajectory.h:94-105); tilts c[6..8] unchanged.
void Trajectory::lammps_to_internal(double *c)
{
    const double zlo = c[4];
    c[5] = (c[5] - c[4]) / 2;
    c[4] = (c[3] - c[2]) / 2;
    c[3] = (c[1] - c[0]) / 2;
    c[1] = c[2];
    c[2] = zlo;
}

// Iterative minimum image, z then y then x, strict '>'
// (lib/include/basetrajectory.h:224-268).
template <bool TRI>
void Trajectory::min_image(double *d, const double *lh, const double *t)
{
    while (std::fabs(d[2]) > lh[2]) {
        if (d[2] < 0.0) {
            d[2] += lh[2] * 2;
            if (TRI) { d[1] += t[2]; d[0] += t[1]; }
        } else {
            d[2] -= lh[2] * 2;
            if (TRI) { d[1] -= t[2]; d[0] -= t[1]; }
        }
    }
    while (std::fabs(d[1]) > lh[1]) {
        if (d[1] < 0.0) {
            d[1] += lh[1] * 2;
            if (TRI) d[0] += t[0];
        } else {
            d[1] -= lh[1] * 2;
            if (TRI) d[0] -= t[0];
        }
    }
    while (std::fabs(d[0]) > lh[0]) {
        if (d[0] < 0.0) d[0] += lh[0] * 2;
        else d[0] -= lh[0] * 2;
    }
}
template void Trajectory::min_image<true>(double *, const double *, const double *);
template void Trajectory::min_image<false>(double *, const double *, const double *);

// ---------------------------------------------------------------------------
// Householder QR of a 3x3 matrix (the published algorithm: reflector
// H = I - tau v v^T with v = [1, essential], beta = -sign(c0) ||x||,
// essential = tail / (c0 - beta), tau = (beta - c0) / beta), evaluated in
// the operation order the reference's linear-algebra library uses for a
// fixed 3x3 matrix, so that the rotated positions carry the same bits.
// ---------------------------------------------------------------------------
namespace {

struct M3 {
    double a[3][3];
};

// Reflector of x[0..n-1] (n = 1..3): returns beta, tau, essential in e[0..n-2].
void make_householder(const double *x, int n, double &beta, double &tau, double *e)
{
    double tail = 0.0;
    if (n == 3) tail = x[1] * x[1] + x[2] * x[2];
    else if (n == 2) tail = x[1] * x[1];
    const double c0 = x[0];
    if (n == 1 || tail <= std::numeric_limits<double>::min()) {
        tau = 0.0;
        beta = c0;
        for (int i = 0; i + 1 < n; ++i) e[i] = 0.0;
        return;
    }
    beta = std::sqrt(c0 * c0 + tail);
    if (c0 >= 0.0) beta = -beta;
    const double den = c0 - beta;
    for (int i = 0; i + 1 < n; ++i) e[i] = x[i + 1] / den;
    tau = (beta - c0) / beta;
}

// Applies H = I - tau [1;e][1;e]^T from the left to the rows r0..2 and
// columns c0..2 of m.
void apply_left(M3 &m, int r0, int c0, const double *e, double tau)
{
    const int rows = 3 - r0;
    if (rows == 1) {
        for (int j = c0; j < 3; ++j) m.a[r0][j] *= (1.0 - tau);
        return;
    }
    if (tau == 0.0) return;
    double tmp[3];
    for (int j = c0; j < 3; ++j) {
        double s = e[0] * m.a[r0 + 1][j];
        if (rows == 3) s = s + e[1] * m.a[r0 + 2][j];
        tmp[j] = s + m.a[r0][j];
    }
    for (int j = c0; j < 3; ++j) m.a[r0][j] -= tau * tmp[j];
    for (int i = 0; i + 1 < rows; ++i) {
        const double te = tau * e[i];
        for (int j = c0; j < 3; ++j) m.a[r0 + 1 + i][j] -= te * tmp[j];
    }
}

}  // namespace

CellQR::CellQR(const double *c)
{
    // cell(i,j) of the reference = c[i + 3j]: its rows are the cell vectors.
    diagonal = c[3] == 0 && c[6] == 0 && c[1] == 0 && c[7] == 0 && c[2] == 0 && c[5] == 0;
    if (diagonal) {
        for (int i = 0; i < 9; ++i) { q[i] = 0.0; r[i] = 0.0; }
        q[0] = q[4] = q[8] = 1.0;
        r[0] = c[0]; r[4] = c[4]; r[8] = c[8];
        return;
    }
    // A = cell^T: A(i,j) = c[3i + j]
    M3 A;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A.a[i][j] = c[3 * i + j];
    double tau[3], ess[3][2];
    for (int k = 0; k < 3; ++k) {
        const int n = 3 - k;
        double x[3], beta;
        for (int i = 0; i < n; ++i) x[i] = A.a[k + i][k];
        make_householder(x, n, beta, tau[k], ess[k]);
        A.a[k][k] = beta;
        for (int i = 0; i + 1 < n; ++i) A.a[k + 1 + i][k] = ess[k][i];
        if (k + 1 < 3) apply_left(A, k, k + 1, ess[k], tau[k]);
    }
    // Q = H0 H1 H2 applied to the identity, last reflector first
    M3 Q;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Q.a[i][j] = i == j ? 1.0 : 0.0;
    for (int k = 2; k >= 0; --k) apply_left(Q, k, k, ess[k], tau[k]);
    // r = upper triangle of A, transposed (lower triangular)
    double R[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = j <= i ? A.a[j][i] : 0.0;
    // positive diagonal: flip column i of r and q where r(i,i) < 0
    for (int i = 0; i < 3; ++i) {
        if (R[i][i] < 0) {
            for (int a = 0; a < 3; ++a) {
                R[a][i] = -R[a][i];
                Q.a[a][i] = -Q.a[a][i];
            }
        }
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            q[3 * i + j] = Q.a[i][j];
            r[3 * i + j] = R[i][j];
        }
}

void CellQR::rotate(double *v) const
{
    double o[3];
    for (int j = 0; j < 3; ++j) o[j] = (v[0] * q[j] + v[1] * q[3 + j]) + v[2] * q[6 + j];
    v[0] = o[0]; v[1] = o[1]; v[2] = o[2];
}

// ---------------------------------------------------------------------------

void Trajectory::wrap_frame(size_t t)
{
    // wrap around the point (lx/2, ly/2, lz/2), as the reference does
    // (basetrajectory.h:145-161: Cell::middle gives the half edges, not xlo+l/2)
    const double *c = boxes_.data() + t * box_stride_;
    static const double zero3[3] = {0.0, 0.0, 0.0};
    const double x0[3] = {c[3], c[4], c[5]};
    for (size_t a = 0; a < natoms_; ++a) {
        double *xa = positions_.data() + (t * natoms_ + a) * 3;
        for (int k = 0; k < 3; ++k) xa[k] = xa[k] - x0[k];
        if (triclinic_) min_image<true>(xa, c + 3, c + 6);
        else min_image<false>(xa, c + 3, zero3);
        for (int k = 0; k < 3; ++k) xa[k] = xa[k] + x0[k];
    }
}

Trajectory::Trajectory(const double *positions, const double *velocities, const int *types,
                       const double *box, size_t nframes, size_t natoms, BoxFormat fmt,
                       bool wrap_pbc, bool save_rotation_matrix)
    : nframes_(nframes), natoms_(natoms), wrap_(wrap_pbc)
{
    if (!positions || !types || !box) throw std::runtime_error("null trajectory buffer");
    if (nframes == 0 || natoms == 0) throw std::runtime_error("empty trajectory");
    std::vector<CellQR> qr;           // one per distinct consecutive cell
    std::vector<size_t> qr_of_frame;  // frame -> index into qr
    if (fmt == BoxFormat::Lammps_ortho || fmt == BoxFormat::Lammps_triclinic) {
        box_stride_ = fmt == BoxFormat::Lammps_triclinic ? 9 : 6;
        triclinic_ = fmt == BoxFormat::Lammps_triclinic;
        boxes_.assign(box, box + nframes * box_stride_);
        for (size_t t = 0; t < nframes; ++t) lammps_to_internal(boxes_.data() + t * box_stride_);
    } else if (fmt == BoxFormat::Cell_vectors) {
        qr_of_frame.resize(nframes);
        for (size_t t = 0; t < nframes; ++t) {
            const double *cur = box + 9 * t;
            // reuse the previous factorisation while the cell does not change
            if (qr.empty() || std::memcmp(cur, box + 9 * (t - 1), 9 * sizeof(double)) != 0)
                qr.emplace_back(cur);
            qr_of_frame[t] = qr.size() - 1;
            if (!qr.back().diagonal) triclinic_ = true;
        }
        box_stride_ = triclinic_ ? 9 : 6;
        boxes_.assign(nframes * box_stride_, 0.0);
        for (size_t t = 0; t < nframes; ++t) {
            const CellQR &f = qr[qr_of_frame[t]];
            double *cel = boxes_.data() + t * box_stride_;
            cel[3] = f.r[0] / 2;
            cel[4] = f.r[4] / 2;
            cel[5] = f.r[8] / 2;
            if (triclinic_) {
                cel[6] = f.r[3];
                cel[7] = f.r[6];
                cel[8] = f.r[7];
            }
        }
    } else {
        throw std::runtime_error("Invalid input cell format");
    }
    positions_.assign(positions, positions + nframes * natoms * 3);
    if (velocities) velocities_.assign(velocities, velocities + nframes * natoms * 3);
    if (triclinic_ && fmt == BoxFormat::Cell_vectors) {
        if (save_rotation_matrix) rotation_.assign(nframes * 9, 0.0);
        for (size_t t = 0; t < nframes; ++t) {
            const CellQR &f = qr[qr_of_frame[t]];
            for (size_t a = 0; a < natoms; ++a) {
                f.rotate(positions_.data() + (t * natoms + a) * 3);
                if (!velocities_.empty()) f.rotate(velocities_.data() + (t * natoms + a) * 3);
            }
            if (save_rotation_matrix)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) rotation_[9 * t + 3 * i + j] = f.q[3 * j + i];
        }
    }
    // dense type ids in sorted order of the raw labels, compared as unsigned
    // integers as the reference does (its label list is std::vector<unsigned>,
    // lib/src/basetrajectory.cpp:60-79), so negative labels sort last
    std::map<unsigned, unsigned> idmap;
    for (size_t a = 0; a < natoms; ++a) idmap.emplace(static_cast<unsigned>(types[a]), 0u);
    unsigned k = 0;
    for (auto &kv : idmap) {
        kv.second = k++;
        types_sorted_.push_back(kv.first);
    }
    type_ids_.resize(natoms);
    for (size_t a = 0; a < natoms; ++a)
        type_ids_[a] = static_cast<int>(idmap[static_cast<unsigned>(types[a])]);
    // Per-frame, per-type centres of mass of the caller's positions (before
    // any rotation or wrapping), running mean over the atoms of each type in
    // atom order, as lib/src/trajectory_numpy.cpp:182,201-222.
    {
        const size_t nt = types_sorted_.size();
        centres_.assign(nframes * nt * 3, 0.0);
        std::vector<int> cont(nt);
        for (size_t t = 0; t < nframes; ++t) {
            std::fill(cont.begin(), cont.end(), 0);
            for (size_t a = 0; a < natoms; ++a) {
                const int k = type_ids_[a];
                cont[k]++;
                for (int c = 0; c < 3; ++c) {
                    double &m = centres_[(t * nt + k) * 3 + c];
                    m += (positions[(t * natoms + a) * 3 + c] - m) / double(cont[k]);
                }
            }
        }
    }
    if (wrap_pbc)
        for (size_t t = 0; t < nframes; ++t) wrap_frame(t);
    static uint64_t counter = 0;
    version_ = ++counter;
}

}  // namespace analisi_gb300
