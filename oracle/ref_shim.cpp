// Reduced Python binding of the reference's own Gofrt path (and its MSD and
// neighbour lists).
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
// reference's unmodified sources lib/src/gofrt.cpp, lib/src/msd.cpp,
// lib/src/neighbour.cpp, lib/src/basetrajectory.cpp and
// lib/src/trajectory_numpy.cpp (see
// oracle/build_ref.sh) into oracle/_ref/pyanalisi_ref*.so.  It exposes the
// classes these paths need, with the constructor and method signatures of the
// full reference binding (pyanalisi/src/pyanalisi.cpp:67-82 for Gofrt,
// :124-152 for MeanSquareDisplacement, :196-236 for Neighbours, :487-527 for
// Trajectory, :528-532 for
// BoxFormat), so that fixtures can be generated by the reference itself and
// the C restatement in oracle/gofr_oracle.c can be pinned against it.
#include <pybind11/pybind11.h>
#include <pybind11/numpy.h>
#include <pybind11/stl.h>
#include "trajectory_numpy.h"
#include "gofrt.h"
#include "msd.h"
#include "neighbour.h"

namespace py = pybind11;

PYBIND11_MODULE(pyanalisi_ref, m) {
    using G = Gofrt<double, Trajectory_numpy>;
    py::class_<Trajectory_numpy>(m, "Trajectory")
        .def(py::init<py::buffer, py::buffer, py::buffer, py::buffer,
                      Trajectory_numpy::BoxFormat, bool, bool>(),
             py::keep_alive<1, 2>(), py::keep_alive<1, 3>(),
             py::keep_alive<1, 4>(), py::keep_alive<1, 5>())
        .def("get_ntypes", &Trajectory_numpy::get_ntypes)
        .def("get_natoms", &Trajectory_numpy::get_natoms)
        .def("get_ntimesteps", &Trajectory_numpy::get_ntimesteps)
        .def("is_triclinic", &Trajectory_numpy::is_triclinic)
        // internal (post-preprocessing) buffers: what the hot path reads
        .def("internal_positions", [](Trajectory_numpy &t) {
            size_t nt = t.get_ntimesteps(), na = t.get_natoms();
            return py::array_t<double>({nt, na, (size_t)3}, t.positions_data());
        })
        .def("internal_boxes", [](Trajectory_numpy &t) {
            size_t nt = t.get_ntimesteps(), st = t.get_box_stride();
            return py::array_t<double>({nt, st}, t.box<false>(0));
        })
        .def("internal_centres", [](Trajectory_numpy &t) {
            size_t nt = t.get_ntimesteps(), ny = t.get_ntypes();
            return py::array_t<double>({nt, ny, (size_t)3}, t.positions_cm<false>(0, 0));
        })
        .def("internal_type_ids", [](Trajectory_numpy &t) {
            size_t na = t.get_natoms();
            py::array_t<int> a(na);
            for (size_t i = 0; i < na; ++i) a.mutable_data()[i] = t.get_type(i);
            return a;
        });
    py::enum_<Trajectory_numpy::BoxFormat>(m, "BoxFormat", py::arithmetic())
        .value("Invalid", Trajectory_numpy::BoxFormat::Invalid)
        .value("CellVectors", Trajectory_numpy::BoxFormat::Cell_vectors)
        .value("LammpsOrtho", Trajectory_numpy::BoxFormat::Lammps_ortho)
        .value("LammpsTriclinic", Trajectory_numpy::BoxFormat::Lammps_triclinic);
    py::class_<G>(m, "Gofrt", py::buffer_protocol())
        .def(py::init<Trajectory_numpy *, double, double, unsigned int, unsigned int,
                      unsigned int, unsigned int, unsigned int, bool>())
        .def("reset", &G::reset)
        .def("getNumberOfExtraTimestepsNeeded", &G::nExtraTimesteps)
        .def("calculate", &G::calculate)
        .def("get_columns_description", &G::get_columns_description)
        .def_buffer([](G &g) -> py::buffer_info {
            return py::buffer_info(g.access_vdata(), sizeof(double),
                                   py::format_descriptor<double>::format(),
                                   g.get_shape().size(), g.get_shape(), g.get_stride());
        });
    using MSDT = MSD<Trajectory_numpy>;
    py::class_<MSDT>(m, "MeanSquareDisplacement", py::buffer_protocol())
        .def(py::init<Trajectory_numpy *, unsigned int, unsigned int, unsigned int, bool, bool,
                      bool>())
        .def("reset", &MSDT::reset)
        .def("getNumberOfExtraTimestepsNeeded", &MSDT::nExtraTimesteps)
        .def("calculate", &MSDT::calculate)
        .def_buffer([](MSDT &g) -> py::buffer_info {
            return py::buffer_info(g.access_vdata(), sizeof(double),
                                   py::format_descriptor<double>::format(),
                                   g.get_shape().size(), g.get_shape(), g.get_stride());
        });
    using NEIGH = Neighbours<Trajectory_numpy, double>;
    py::class_<NEIGH>(m, "Neighbours")
        .def(py::init<Trajectory_numpy *, typename NEIGH::ListSpec>(), py::keep_alive<1, 2>())
        .def("calculate_neigh", &NEIGH::update_neigh)
        .def("get_sann", [](NEIGH &n, size_t iatom, size_t jtype) {
            auto it = n.get_sann_r(iatom, jtype);
            return py::array_t<double>({(ssize_t)it.size(), (ssize_t)4}, (const double *)it.begin());
        })
        .def("get_sann_idx", [](NEIGH &n, size_t iatom, size_t jtype) {
            auto it = n.get_sann(iatom, jtype);
            return py::array_t<size_t>({(ssize_t)it.size()}, it.begin());
        })
        .def("get_neigh", [](NEIGH &n, size_t iatom, size_t jtype) {
            auto it = n.get_neigh_r(iatom, jtype);
            return py::array_t<double>({(ssize_t)it.size(), (ssize_t)4}, (const double *)it.begin());
        })
        .def("get_neigh_idx", [](NEIGH &n, size_t iatom, size_t jtype) {
            auto it = n.get_neigh(iatom, jtype);
            return py::array_t<size_t>({(ssize_t)it.size()}, it.begin());
        });
}
