// Python module `pyanalisi` of analisi_gb300: the reference's Gofrt path API
// (pyanalisi/src/pyanalisi.cpp:67-82 for Gofrt, :124-152 for
// MeanSquareDisplacement, :196-236 for Neighbours, :487-532 for Trajectory and
// BoxFormat) with the GB300 engine behind it.
//
//   import pyanalisi        # analisi_gb300/_build on sys.path
//   t = pyanalisi.Trajectory(pos, vel, types, box, pyanalisi.BoxFormat.CellVectors, False, False)
//   g = pyanalisi.Gofrt(t, rmin, rmax, nbin, tmax, nthreads, skip, every, debug)
//   g.reset(n); g.calculate(primo); a = np.array(g, copy=True)
//
// Argument checks and their messages follow lib/src/trajectory_numpy.cpp:20-118.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cstring>
#include <memory>

#include "gofrt.h"
#include "lammps_file.h"
#include "msd.h"
#include "neighbour.h"
#include "traj_window.h"
#include "trajectory.h"

namespace py = pybind11;
using analisi_gb300::BoxFormat;
using analisi_gb300::Trajectory;
using analisi_gb300::TrajWindow;
using GofrtT = analisi_gb300::Gofrt<double, Trajectory>;
using GofrtW = analisi_gb300::Gofrt<double, TrajWindow>;
using MsdT = analisi_gb300::MeanSquareDisplacement<Trajectory>;
using NeighT = analisi_gb300::Neighbours<Trajectory, double>;

namespace {

template <typename T>
bool has_no_stride(const py::buffer_info &b)
{
    ssize_t stride = sizeof(T);
    for (int i = (int)b.ndim - 1; i >= 0; --i) {
        if (b.strides[i] != stride) return false;
        stride *= b.shape[i];
    }
    return true;
}

std::unique_ptr<Trajectory> make_trajectory(py::buffer pos, py::buffer vel, py::buffer types,
                                            py::buffer box, BoxFormat fmt, bool wrap,
                                            bool save_rot)
{
    py::buffer_info ip = pos.request(), iv = vel.request(), it = types.request(),
                    ib = box.request();
    if (ip.ndim != 3) throw std::runtime_error("Wrong number of dimension of position array (must be 3)");
    if (iv.ndim != 3) throw std::runtime_error("Wrong number of dimension of velocities array (must be 3)");
    if (ip.shape[2] != 3)
        throw std::runtime_error("Wrong number of cartesian components in the third dimension of positions array");
    if (iv.shape[2] != 3)
        throw std::runtime_error("Wrong number of cartesian components in the third dimension of velocities array");
    for (int i = 0; i < 3; ++i)
        if (ip.shape[i] != iv.shape[i])
            throw std::runtime_error("Shape of positions and velocities array is different");
    if (it.ndim != 1) throw std::runtime_error("Wrong number of dimension of types array (must be 1)");
    if (it.shape[0] != ip.shape[1]) throw std::runtime_error("Wrong size of the type array");
    if (fmt == BoxFormat::Cell_vectors) {
        if (ib.ndim != 3)
            throw std::runtime_error("Wrong number of dimensions of box array (must be 3) for cell matrix format");
        if (ib.shape[0] != ip.shape[0] || ib.shape[1] != 3 || ib.shape[2] != 3)
            throw std::runtime_error("Wrong shape of box array: must be (nsteps, 3, 3) for matrix format");
    } else {
        if (ib.ndim != 2)
            throw std::runtime_error("Wrong number of dimensions of box array (must be 2 for lammps ortho/triclinic cell format)");
        if (ib.shape[0] != ip.shape[0])
            throw std::runtime_error("Wrong shape of box array: first dimension must be nsteps");
        if (fmt == BoxFormat::Lammps_ortho && ib.shape[1] != 6)
            throw std::runtime_error("Wrong shape of box array: must be (:, 6) for orthogonal lammps cell format");
        if (fmt == BoxFormat::Lammps_triclinic && ib.shape[1] != 9)
            throw std::runtime_error("Wrong shape of box array: must be (:, 9) for triclinic lammps cell format");
    }
    if (ib.format != py::format_descriptor<double>::format())
        throw std::runtime_error("Format of box array should be double");
    if (it.format != py::format_descriptor<int>::format())
        throw std::runtime_error("Format of types array should be int (" +
                                 py::format_descriptor<int>::format() + ") while it was " +
                                 it.format);
    if (iv.format != py::format_descriptor<double>::format())
        throw std::runtime_error("Format of velocities array should be double");
    if (ip.format != py::format_descriptor<double>::format())
        throw std::runtime_error("Format of positions array should be double");
    if (!has_no_stride<double>(ib)) throw std::runtime_error("Unsupported stride in box array");
    if (!has_no_stride<int>(it)) throw std::runtime_error("Unsupported stride in types array");
    if (!has_no_stride<double>(iv)) throw std::runtime_error("Unsupported stride in vel array");
    if (!has_no_stride<double>(ip)) throw std::runtime_error("Unsupported stride in pos array");
    if (fmt == BoxFormat::Invalid) throw std::runtime_error("Invalid input cell format");
    return std::make_unique<Trajectory>(
        static_cast<const double *>(ip.ptr), static_cast<const double *>(iv.ptr),
        static_cast<const int *>(it.ptr), static_cast<const double *>(ib.ptr),
        (size_t)ip.shape[0], (size_t)ip.shape[1], fmt, wrap, save_rot);
}

py::array_t<double> copy3(const double *p, size_t a, size_t b, size_t c)
{
    py::array_t<double> out({a, b, c});
    if (a * b * c != 0) std::memcpy(out.mutable_data(), p, sizeof(double) * a * b * c);
    return out;
}

// The reference's Gofrt binding (pyanalisi/src/pyanalisi.cpp:66-82) for a
// trajectory type T: `Gofrt` over Trajectory, `Gofrt_lammps` over Traj.
template <class G, class T>
void define_gofrt(py::module &m, const char *name)
{
    py::class_<G>(m, name, py::buffer_protocol())
        .def(py::init<T *, double, double, unsigned int, unsigned int, unsigned int,
                      unsigned int, unsigned int, bool>(),
             py::arg("trajectory"), py::arg("rmin"), py::arg("rmax"), py::arg("nbin"),
             py::arg("tmax") = 0, py::arg("nthreads") = 0, py::arg("skip") = 1,
             py::arg("every") = 1, py::arg("debug") = false, py::keep_alive<1, 2>(),
             R"doc(calculates g(r) and, in general, g(r,t) on the GPU

Parameters
----------
Trajectory instance, rmin, rmax, nbin, maximum time lag, number of threads
(the reference's atom split; its per-thread sums are reproduced exactly),
time skip, every time, debug flag)doc")
        .def("reset", &G::reset)
        .def("getNumberOfExtraTimestepsNeeded", &G::nExtraTimesteps)
        .def("calculate", [](G &g, size_t primo) {
            py::gil_scoped_release release;
            g.calculate(primo);
        })
        .def("get_columns_description", &G::get_columns_description)
        .def("set_device_budget", &G::set_device_budget,
             "frames beyond this many device bytes are streamed through the GPU in chunks "
             "of origins (0: all resident)")
        .def("set_kernel", &G::set_kernel,
             "0 auto (FP32 + FP64 edge recheck), 1 FP32 forced, 2 plain FP64")
        .def("last_stats", [](G &g) {
            gofr_stats s = g.last_stats();
            py::dict d;
            d["pairs"] = s.pairs;
            d["evaluated"] = s.evaluated;
            d["candidates"] = s.candidates;
            d["rechecks"] = s.rechecks;
            d["kernel_ms"] = s.kernel_ms;
            d["total_ms"] = s.total_ms;
            d["kernel_used"] = s.kernel_used;
            d["wrap_checked"] = s.wrap_checked;
            d["err_bound_d2"] = s.err_bound_d2;
            return d;
        })
        .def_buffer([](G &g) -> py::buffer_info {
            return py::buffer_info(g.access_vdata(), sizeof(double),
                                   py::format_descriptor<double>::format(), g.get_shape().size(),
                                   g.get_shape(), g.get_stride());
        });
}

}  // namespace

PYBIND11_MODULE(pyanalisi, m)
{
    m.doc() = "analisi's Gofrt (van Hove g(r,t)) on the GB300 engine";

    py::enum_<BoxFormat>(m, "BoxFormat", py::arithmetic())
        .value("Invalid", BoxFormat::Invalid)
        .value("CellVectors", BoxFormat::Cell_vectors)
        .value("LammpsOrtho", BoxFormat::Lammps_ortho)
        .value("LammpsTriclinic", BoxFormat::Lammps_triclinic);

    py::class_<Trajectory>(m, "Trajectory")
        .def(py::init(&make_trajectory), py::arg("positions"), py::arg("velocities"),
             py::arg("types"), py::arg("box"), py::arg("box_format") = BoxFormat::Cell_vectors,
             py::arg("wrap") = false, py::arg("save_rotation_matrix") = false,
             R"doc(Parameters
----------
positions (double) array (ntimesteps, natoms, 3)
velocities (double) array (ntimesteps, natoms, 3)
types (int) array (natoms)
box (double): (ntimesteps, 3, 3) cell vectors as columns, or (ntimesteps, 6|9) lammps rows
format of the box (BoxFormat)
wrap atoms inside the cell using pbc
save rotation matrix if triclinic format is used and a rotation is needed)doc")
        .def("get_positions_copy", [](Trajectory &t) {
            return copy3(t.positions_data(), t.get_ntimesteps(), t.get_natoms(), 3);
        })
        .def("get_velocities_copy", [](Trajectory &t) {
            if (!t.velocity_data()) return py::array_t<double>();
            return copy3(t.velocity_data(), t.get_ntimesteps(), t.get_natoms(), 3);
        })
        .def("get_box_copy", [](Trajectory &t) {
            py::array_t<double> out({t.get_ntimesteps(), t.get_box_stride()});
            std::memcpy(out.mutable_data(), t.box(0),
                        sizeof(double) * t.get_ntimesteps() * t.get_box_stride());
            return out;
        })
        .def("get_rotation_matrix", [](Trajectory &t) {
            const auto &r = t.rotation_matrix();
            if (r.empty()) return py::array_t<double>();
            return copy3(r.data(), t.get_ntimesteps(), 3, 3);
        })
        .def("get_centres_copy", [](Trajectory &t) {
            return copy3(t.centres_data(), t.get_ntimesteps(), t.get_ntypes(), 3);
        }, "per-frame, per-type centres of mass (the reference's positions_cm)")
        .def("get_type", &Trajectory::get_type, "get the type used for the internal representation")
        .def("get_type_ids", [](Trajectory &t) {
            py::array_t<int> out(t.get_natoms());
            std::memcpy(out.mutable_data(), t.type_ids(), sizeof(int) * t.get_natoms());
            return out;
        })
        .def("get_ntypes", &Trajectory::get_ntypes)
        .def("get_natoms", &Trajectory::get_natoms)
        .def("is_triclinic", &Trajectory::is_triclinic)
        .def("get_nloaded_timesteps", &Trajectory::get_nloaded_timesteps)
        .def("getNtimesteps", &Trajectory::get_ntimesteps)
        .def("get_current_timestep", [](Trajectory &) { return (ssize_t)0; })
        .def("getWrapPbc", &Trajectory::get_pbc_wrap)
        .def("data_version", &Trajectory::data_version,
             "changes whenever the internal buffers change (device copies follow it)");

    define_gofrt<GofrtT, Trajectory>(m, "Gofrt");

    // the reference's memory-mapped trajectory (pyanalisi/src/pyanalisi.cpp:376-418)
    py::class_<TrajWindow>(m, "Traj", py::buffer_protocol())
        .def(py::init<std::string>(), R"doc(Parameters
----------
name of the binary file to open)doc")
        .def("setWrapPbc", &TrajWindow::set_pbc_wrap,
             "wrap all the atomic coordinates inside the simulation box (True/False)")
        .def("setAccessWindowSize", [](TrajWindow &t, int ts) {
            return ts > 0 ? t.set_data_access_block_size((size_t)ts) : 0;
        }, "sets the number of frames of the read window; 1 success, 0 failure")
        .def("setAccessStart", [](TrajWindow &t, int ts) {
            return ts >= 0 ? t.set_access_at((size_t)ts) : 0;
        }, "reads the window starting at this frame; 1 success, 2 beyond the end of the file")
        .def("serving_pos", &TrajWindow::serving_pos)
        .def("toggle_pos_vel", &TrajWindow::toggle_pos_vel)
        .def("get_positions_copy", [](TrajWindow &t) {
            return copy3(t.positions_data(), t.window_frames(), t.get_natoms(), 3);
        })
        .def("get_velocities_copy", [](TrajWindow &t) {
            return copy3(t.velocity_data(), t.window_frames(), t.get_natoms(), 3);
        })
        .def("get_box_copy", [](TrajWindow &t) {
            const size_t st = t.get_box_stride(), n = t.window_frames();
            py::array_t<double> b({n, st});
            if (n) std::memcpy(b.mutable_data(), t.box(0), sizeof(double) * n * st);
            return b;
        })
        .def("get_type_ids", [](TrajWindow &t) {
            return py::array_t<int>(t.get_natoms(), t.type_ids());
        })
        .def("get_ntypes", &TrajWindow::get_ntypes)
        .def("get_natoms", &TrajWindow::get_natoms)
        .def("is_triclinic", &TrajWindow::is_triclinic)
        .def("get_nloaded_timesteps", &TrajWindow::get_nloaded_timesteps)
        .def("getNtimesteps", &TrajWindow::get_ntimesteps)
        .def("get_current_timestep", &TrajWindow::window_start)
        .def("getWrapPbc", &TrajWindow::get_pbc_wrap)
        .def("get_lammps_timesteps", [](TrajWindow &t) {
            const auto &v = t.lammps_timesteps();
            return py::array_t<long long>(v.size(), reinterpret_cast<const long long *>(v.data()));
        })
        .def_buffer([](TrajWindow &t) -> py::buffer_info {
            const ssize_t n = (ssize_t)t.window_frames(), na = (ssize_t)t.get_natoms();
            const double *d = t.serving_pos() ? t.positions_data() : t.velocity_data();
            return py::buffer_info(const_cast<double *>(d), sizeof(double),
                                   py::format_descriptor<double>::format(), 3, {n, na, (ssize_t)3},
                                   {(ssize_t)(na * 3 * sizeof(double)),
                                    (ssize_t)(3 * sizeof(double)), (ssize_t)sizeof(double)});
        });
    define_gofrt<GofrtW, TrajWindow>(m, "Gofrt_lammps");

    py::class_<MsdT>(m, "MeanSquareDisplacement", py::buffer_protocol())
        .def(py::init<Trajectory *, unsigned int, unsigned int, unsigned int, bool, bool, bool>(),
             py::arg("trajectory"), py::arg("skip") = 1, py::arg("tmax") = 0,
             py::arg("nthreads") = 0, py::arg("center_of_mass") = false,
             py::arg("in_center_of_mass_frame") = false, py::arg("debug") = false,
             py::keep_alive<1, 2>(),
             R"doc(mean square displacement on the GPU

Parameters
----------
Trajectory instance
time skip for the average computation
max time
number of threads (no effect: the GPU computes every lag)
calculate center of mass MSD
calculate for each atomic specie the atomic msd in the center of mass reference system of that specie
debug flag)doc")
        .def("reset", &MsdT::reset)
        .def("getNumberOfExtraTimestepsNeeded", &MsdT::nExtraTimesteps)
        .def("calculate", [](MsdT &m, size_t primo) {
            py::gil_scoped_release release;
            m.calculate(primo);
        })
        .def("last_stats", [](MsdT &m) {
            gofr_stats s = m.last_stats();
            py::dict d;
            d["displacements"] = s.pairs;
            d["kernel_ms"] = s.kernel_ms;
            d["total_ms"] = s.total_ms;
            return d;
        })
        .def_buffer([](MsdT &m) -> py::buffer_info {
            return py::buffer_info(m.access_vdata(), sizeof(double),
                                   py::format_descriptor<double>::format(), m.get_shape().size(),
                                   m.get_shape(), m.get_stride());
        })
        .def("__enter__", [](MsdT &m) -> MsdT & { return m; }, py::return_value_policy::reference)
        .def("__exit__", [](MsdT &, py::object, py::object, py::object) {});

    py::class_<NeighT>(m, "Neighbours")
        .def(py::init<Trajectory *, typename NeighT::ListSpec>(), py::arg("trajectory"),
             py::arg("nneigh_cut2_skin2"), py::keep_alive<1, 2>(),
             "neighbour lists: [(max neighbours, cutoff^2, skin^2)] for each atomic type")
        .def("calculate_neigh", [](NeighT &n, size_t timestep, bool sort) {
            py::gil_scoped_release release;
            n.update_neigh(timestep, sort);
        })
        .def("get_sann", [](NeighT &n, size_t iatom, size_t jtype) {
            auto it = n.get_sann_r(iatom, jtype);
            return py::array_t<double>({(ssize_t)it.size(), (ssize_t)4},
                                       reinterpret_cast<const double *>(it.begin()));
        })
        .def("get_sann_idx", [](NeighT &n, size_t iatom, size_t jtype) {
            auto it = n.get_sann(iatom, jtype);
            return py::array_t<size_t>({(ssize_t)it.size()}, it.begin());
        })
        .def("get_neigh", [](NeighT &n, size_t iatom, size_t jtype) {
            auto it = n.get_neigh_r(iatom, jtype);
            return py::array_t<double>({(ssize_t)it.size(), (ssize_t)4},
                                       reinterpret_cast<const double *>(it.begin()));
        })
        .def("get_neigh_idx", [](NeighT &n, size_t iatom, size_t jtype) {
            auto it = n.get_neigh(iatom, jtype);
            return py::array_t<size_t>({(ssize_t)it.size()}, it.begin());
        });

    m.def("read_lammps_binary", [](const std::string &path) {
        analisi_gb300::LammpsFrames f = analisi_gb300::read_lammps_binary(path);
        py::dict d;
        d["positions"] = copy3(f.positions.data(), f.nframes, f.natoms, 3);
        d["velocities"] = copy3(f.velocities.data(), f.nframes, f.natoms, 3);
        const size_t st = f.triclinic ? 9 : 6;
        py::array_t<double> b({f.nframes, st});
        std::memcpy(b.mutable_data(), f.boxes.data(), sizeof(double) * f.nframes * st);
        d["boxes"] = b;
        d["types"] = py::array_t<int>(f.types.size(), f.types.data());
        d["timesteps"] = py::array_t<long long>(f.timesteps.size(),
                                                reinterpret_cast<const long long *>(f.timesteps.data()));
        d["triclinic"] = f.triclinic;
        return d;
    }, "reads analisi's binary trajectory format (the CLI's -i input)");
    m.def("info", []() { return std::string("analisi_gb300: Gofrt on GB300 (sm_103a)"); });
    m.def("has_mmap", []() { return true; });
}
