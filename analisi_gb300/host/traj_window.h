// TrajWindow: the reference's memory-mapped trajectory (lib/include/trajectory.h,
// lib/src/trajectory.cpp), the `Traj` of its Python module
// (pyanalisi/src/pyanalisi.cpp:376-418): a binary trajectory file mapped into
// memory, of which a window of frames is decoded and preprocessed at a time
// (set_data_access_block_size / set_access_at), so a file larger than memory
// can be analysed.  A g(r,t) calculation over it (Gofrt_lammps) loads the
// window its origins and lags need, as the reference's accessors load one on
// demand (lib/include/trajectory.h:41-72), and copies only that window to the
// GPU.
#pragma once
#include <algorithm>
#include <cstdint>
#include <set>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "lammps_file.h"
#include "trajectory.h"

namespace analisi_gb300 {

class TrajWindow {
public:
    // lib/include/basetrajectory.h:78
    enum Errori { non_inizializzato = 0, Ok = 1, oltre_fine_file = 2 };

    explicit TrajWindow(const std::string &filename) : file_(new LammpsMmap(filename))
    {
        // types are the first frame's labels (known before any window is read)
        ntypes_ = std::set<int>(file_->types().begin(), file_->types().end()).size();
    }

    // The window is rebuilt (wrapped or not) at the next set_access_at.
    void set_pbc_wrap(bool wrap)
    {
        if (wrap != wrap_) {
            wrap_ = wrap;
            window_.reset();
        }
    }
    bool get_pbc_wrap() const { return wrap_; }

    int set_data_access_block_size(size_t n)
    {
        if (n == 0) return non_inizializzato;
        if (n != block_) {
            block_ = n;
            window_.reset();
        }
        return Ok;
    }

    // Frames [timestep, timestep + block) decoded, preprocessed (the LAMMPS
    // rows to the internal box, wrapped when asked) and kept as the window.
    int set_access_at(size_t timestep)
    {
        if (window_ && timestep == start_) return Ok;
        if (timestep + block_ > file_->nframes()) return oltre_fine_file;
        load(timestep, block_);
        return Ok;
    }

    // Makes frames [first, first + count) resident in the window: nothing if
    // they already are, else the window is moved to start at `first` (and
    // grown to `count` frames if the block is shorter).  Throws the
    // reference's message when the file ends before.
    void ensure_window(size_t first, size_t count)
    {
        if (first + count > file_->nframes())
            throw std::runtime_error(
                "trajectory is too short for this kind of calculation. Select a different "
                "starting timestep or lower the size of the average or the lenght of the time "
                "lag");
        if (window_ && first >= start_ && first + count <= start_ + window_->get_ntimesteps())
            return;
        load(first, std::max(count, block_));
    }

    // the trajectory interface the calculations use (the window)
    size_t window_start() const { return start_; }
    size_t window_frames() const { return window_ ? window_->get_ntimesteps() : 0; }
    size_t get_ntimesteps() const { return file_->nframes(); }
    size_t get_nloaded_timesteps() const { return window_frames(); }
    size_t get_natoms() const { return file_->natoms(); }
    size_t get_ntypes() const { return ntypes_; }
    std::vector<unsigned int> get_types() const { return need().get_types(); }
    bool is_triclinic() const { return file_->triclinic(); }
    size_t get_box_stride() const { return need().get_box_stride(); }
    const double *positions_data() const { return need().positions_data(); }
    const double *velocity_data() const { return need().velocity_data(); }
    const double *box(size_t t) const { return need().box(t); }
    const int *type_ids() const { return need().type_ids(); }
    uint64_t data_version() const { return window_ ? window_->data_version() : 0; }
    const Trajectory &window() const { return need(); }
    const std::vector<int64_t> &lammps_timesteps() const { return file_->timesteps(); }
    // which of the window's arrays the Python buffer protocol serves
    bool serving_pos() const { return serving_pos_; }
    void toggle_pos_vel() { serving_pos_ = !serving_pos_; }

private:
    const Trajectory &need() const
    {
        if (!window_)
            throw std::runtime_error("no frames loaded: call setAccessWindowSize and "
                                     "setAccessStart first");
        return *window_;
    }

    void load(size_t first, size_t count)
    {
        LammpsFrames f = file_->read(first, count);
        window_.reset(new Trajectory(
            f.positions.data(), f.velocities.data(), f.types.data(), f.boxes.data(), f.nframes,
            f.natoms, f.triclinic ? BoxFormat::Lammps_triclinic : BoxFormat::Lammps_ortho, wrap_,
            false));
        start_ = first;
    }

    std::unique_ptr<LammpsMmap> file_;
    std::unique_ptr<Trajectory> window_;
    size_t block_ = 1, start_ = 0, ntypes_ = 0;
    bool wrap_ = false, serving_pos_ = true;
};

}  // namespace analisi_gb300
