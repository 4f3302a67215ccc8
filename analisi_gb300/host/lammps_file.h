// Reader of analisi's binary trajectory files (the input of the CLI, -i).
//
// Format (restated from lib/include/lammps_struct.h:31-260 and
// lib/src/trajectory.cpp:261-345,450-690): a sequence of frames, each a
// header followed by `nchunk` chunks of {int n_double; double data[n_double]}
// where every atom is 8 doubles {id, type, x, y, z, vx, vy, vz}.  Headers:
//   classic:     int64 timestep (>= 0), int64 natoms, int triclinic, int bc[6],
//                double box[6] (xlo,xhi,ylo,yhi,zlo,zhi), [double xy,xz,yz if
//                triclinic], int doubles_per_atom, int nchunk
//   LAMMPS 2020: int64 -len, char magic[len], int endian, int revision,
//                int64 timestep, int64 natoms, int triclinic, int bc[6],
//                double box[6], [double tilt[3]], int doubles_per_atom,
//                (revision > 1: int ulen, char unit_style[ulen], char time_flag,
//                [double time], int clen, char columns[clen]), int nchunk
// Atoms are stored in the order of first appearance in the first frame, each
// later frame's atoms placed by id (lib/src/trajectory.cpp:630-660); types
// come from the first frame, rounded.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace analisi_gb300 {

struct LammpsFrames {
    size_t nframes = 0, natoms = 0;
    bool triclinic = false;
    std::vector<double> positions;   // [nframes][natoms][3]
    std::vector<double> velocities;  // [nframes][natoms][3]
    std::vector<double> boxes;       // [nframes][6|9] lammps rows xlo,xhi,ylo,yhi,zlo,zhi[,xy,xz,yz]
    std::vector<int> types;          // [natoms] raw labels
    std::vector<int64_t> timesteps;  // LAMMPS timestep of each frame
};

// A binary trajectory file mapped into memory (mmap, read-only) with an
// index of its frames, built by walking the headers and chunk sizes once
// (the reference's Trajectory, lib/src/trajectory.cpp:261-345,450-690, which
// also maps the file and indexes it).  Frames are decoded on request, a
// window at a time, so the file is never copied whole.
class LammpsMmap {
public:
    explicit LammpsMmap(const std::string &path);  // throws std::runtime_error
    ~LammpsMmap();
    LammpsMmap(const LammpsMmap &) = delete;
    LammpsMmap &operator=(const LammpsMmap &) = delete;

    size_t nframes() const { return offsets_.size(); }
    size_t natoms() const { return natoms_; }
    bool triclinic() const { return triclinic_; }
    const std::vector<int> &types() const { return types_; }  // raw labels (first frame)
    const std::vector<int64_t> &timesteps() const { return steps_; }
    // Decodes frames [first, first + count) (atoms in first-frame order).
    LammpsFrames read(size_t first, size_t count) const;

private:
    const char *data_ = nullptr;
    size_t size_ = 0;
    size_t natoms_ = 0;
    bool triclinic_ = false;
    std::vector<size_t> offsets_;     // byte offset of each frame's header
    std::vector<int64_t> steps_;
    std::vector<int> types_;
    std::vector<long long> ids_;      // atom id of each first-frame slot
};

// Throws std::runtime_error on a malformed file.
LammpsFrames read_lammps_binary(const std::string &path);

// Writes frames in the classic format (one chunk per frame); ids are 1..N.
void write_lammps_binary(const std::string &path, const LammpsFrames &f);

}  // namespace analisi_gb300
