// Host-side trajectory of the GB300 Gofrt path.
//
// Restates the preprocessing of the reference's Trajectory_numpy
// (lib/src/trajectory_numpy.cpp:7-199) that fixes the FP64 values the g(r,t)
// hot path reads: box conversion to the internal format
// {xlo, ylo, zlo, lx/2, ly/2, lz/2[, xy, xz, yz]} (lib/include/basetrajectory.h:
// 94-105), the QR of non-diagonal cell vectors with the rotation of the
// positions (lib/include/triclinic.h:10-37), the dense type ids
// (lib/src/basetrajectory.cpp:52-89) and the optional pbc wrap
// (lib/include/basetrajectory.h:145-161).  The device engine then consumes
// exactly these buffers (positions_data(), box(0), type_ids()).
//
// Differences from the reference, on purpose:
//  * buffers are always owned copies (the reference aliases the input when no
//    copy is needed; values are identical);
//  * with BoxFormat::Lammps_triclinic and wrap=false the reference allocates
//    its internal positions but never copies the input into them
//    (lib/src/trajectory_numpy.cpp:185-213) and computes on uninitialised
//    memory; here the input is copied;
//  * centre-of-mass buffers are not built (nothing on the g(r,t) path reads them).
#pragma once
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace analisi_gb300 {

// Same enumerators and order as the reference's BaseTrajectory::BoxFormat
// (lib/include/basetrajectory.h:50).
enum class BoxFormat { Lammps_ortho = 0, Lammps_triclinic = 1, Cell_vectors = 2, Invalid = 3 };

class Trajectory {
public:
    // positions, velocities: [nframes][natoms][3]; types: [natoms] raw labels;
    // box: [nframes][3][3] (Cell_vectors, columns are the cell vectors),
    // [nframes][6] (Lammps_ortho: xlo,xhi,ylo,yhi,zlo,zhi) or [nframes][9]
    // (Lammps_triclinic: ... ,xy,xz,yz).  velocities may be null.
    Trajectory(const double *positions, const double *velocities, const int *types,
               const double *box, size_t nframes, size_t natoms, BoxFormat fmt,
               bool wrap_pbc = false, bool save_rotation_matrix = false);

    size_t get_natoms() const { return natoms_; }
    size_t get_ntimesteps() const { return nframes_; }
    size_t get_nloaded_timesteps() const { return nframes_; }
    size_t get_ntypes() const { return types_sorted_.size(); }
    std::vector<unsigned int> get_types() const { return types_sorted_; }
    unsigned int get_type(size_t atom) const
    {
        if (atom < natoms_) return static_cast<unsigned>(type_ids_[atom]);
        throw std::runtime_error("Atom index out of range\n");
    }
    bool is_triclinic() const { return triclinic_; }
    size_t get_box_stride() const { return box_stride_; }
    bool get_pbc_wrap() const { return wrap_; }

    const double *positions_data() const { return positions_.data(); }
    const double *velocity_data() const { return velocities_.data(); }
    const double *box(size_t t) const { return boxes_.data() + t * box_stride_; }
    const double *positions(size_t t, size_t atom) const
    {
        return positions_.data() + (t * natoms_ + atom) * 3;
    }
    const int *type_ids() const { return type_ids_.data(); }
    // [T][ntypes][3] centres of mass of each type (the reference's positions_cm)
    const double *centres_data() const { return centres_.data(); }
    // [nframes][3][3] rotation applied to positions (only for non-diagonal
    // cell vectors with save_rotation_matrix), else empty.
    const std::vector<double> &rotation_matrix() const { return rotation_; }
    // Changes whenever the internal buffers change (engines re-upload on change).
    uint64_t data_version() const { return version_; }

    // helpers shared with the CLI front end
    static void lammps_to_internal(double *c);
    template <bool TRI>
    static void min_image(double *delta, const double *l_half, const double *xy_xz_yz);

private:
    void wrap_frame(size_t t);

    size_t nframes_ = 0, natoms_ = 0, box_stride_ = 6;
    bool triclinic_ = false, wrap_ = false;
    std::vector<double> positions_, velocities_, boxes_, rotation_, centres_;
    std::vector<int> type_ids_;
    std::vector<unsigned int> types_sorted_;
    uint64_t version_ = 0;
};

// Householder QR of a 3x3 cell (TriclinicLammpsCell, lib/include/triclinic.h:10-37):
// r lower triangular with positive diagonal ("LAMMPS" form), q orthogonal,
// both row-major [3][3]; cell is [3][3] row-major with the cell vectors as columns.
struct CellQR {
    double q[9], r[9];
    bool diagonal;
    explicit CellQR(const double *cell);
    void rotate(double *v) const;  // v <- v * q (row vector)
};

}  // namespace analisi_gb300
