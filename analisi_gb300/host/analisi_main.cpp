// `analisi` command line, g(r,t) and mean-square-displacement branches, on
// the GB300 engine.
//
//   analisi -i traj.bin -g NBIN -F RMIN RMAX [-S TMAX] [-s SKIP] [-e EVERY]
//           [-N THREADS] [-B BLOCKS] [-d]
//   analisi -i traj.bin -q|-Q|--mean-square-displacement-self [-S TMAX] [-s SKIP]
//           [-N THREADS] [-B BLOCKS] [-d]
//
// Same options, defaults and output as the reference's gofr branch
// (analisi/main.cpp:162-232 for the options, :552-584 for the computation and
// the printout): the trajectory is read with pbc wrapping on, split into
// BLOCKS block averages, and each (lag, bin) row prints the mean and variance
// of every channel.  -N is the reference's thread count: the per-thread sums
// it implies are reproduced exactly.  The MSD branch (analisi/main.cpp:520-551)
// reads the trajectory as it is (no wrapping), block-averages
// MSD(skip, TMAX, N, cm, self, dump) and prints, per lag, mean and variance of
// every type (and of every type's centre of mass with -Q).  Options of the
// reference's other analyses are rejected.
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "blockaverage.h"
#include "gofrt.h"
#include "lammps_file.h"
#include "msd.h"
#include "trajectory.h"

using namespace analisi_gb300;

namespace {

void usage()
{
    std::cerr << "analisi (GB300 g(r,t) engine)\n"
                 "  -i, --input FILE        binary trajectory (id type xu yu zu vx vy vz)\n"
                 "  -g, --gofrt NBIN        histogram bins of g(r,t)\n"
                 "  -F, --factors RMIN RMAX distance range of the histogram\n"
                 "  -S, --stop TMAX         maximum time lag (0: as long as possible)\n"
                 "  -s, --skip SKIP         stride between time origins\n"
                 "  -e, --every EVERY       stride between time lags\n"
                 "  -N, --thread N          threads of the reference's split (default OMP_NUM_THREADS or 2)\n"
                 "  -B, --blocknumber B     blocks of the average (default 20)\n"
                 "  -q, --mean-square-displacement       atomic mean square displacement\n"
                 "  -Q, --mean-square-displacement-cm    and of each type's centre of mass\n"
                 "      --mean-square-displacement-self  in each type's centre-of-mass frame\n"
                 "  -d, --dump-block        append every block's buffer to gofrt.dump / msd.dump\n";
}

}  // namespace

int main(int argc, char **argv)
{
    int nthreads = 2;
    if (const char *o = std::getenv("OMP_NUM_THREADS")) {
        const int v = std::atoi(o);
        if (v > 0) nthreads = v;
    }
    std::string input;
    unsigned nbin = 0;
    std::vector<double> factors;
    int tmax = 0, skip = 1, every = 1, blocks = 20;
    bool dump = false, msd = false, msd_cm = false, msd_self = false;
    try {
        for (int a = 1; a < argc; ++a) {
            const std::string k = argv[a];
            auto need = [&](int n) {
                if (a + n >= argc) throw std::runtime_error("missing value for option " + k);
            };
            if (k == "-i" || k == "--input") { need(1); input = argv[++a]; }
            else if (k == "-g" || k == "--gofrt") { need(1); nbin = (unsigned)std::stoul(argv[++a]); }
            else if (k == "-F" || k == "--factors") {
                while (a + 1 < argc && (argv[a + 1][0] != '-' ||
                                        (argv[a + 1][1] >= '0' && argv[a + 1][1] <= '9') ||
                                        argv[a + 1][1] == '.'))
                    factors.push_back(std::stod(argv[++a]));
            } else if (k == "-S" || k == "--stop") { need(1); tmax = std::stoi(argv[++a]); }
            else if (k == "-s" || k == "--skip") { need(1); skip = std::stoi(argv[++a]); }
            else if (k == "-e" || k == "--every") { need(1); every = std::stoi(argv[++a]); }
            else if (k == "-N" || k == "--thread") { need(1); nthreads = std::stoi(argv[++a]); }
            else if (k == "-B" || k == "--blocknumber") { need(1); blocks = std::stoi(argv[++a]); }
            else if (k == "-d" || k == "--dump-block") dump = true;
            else if (k == "-q" || k == "--mean-square-displacement") msd = true;
            else if (k == "-Q" || k == "--mean-square-displacement-cm") msd_cm = true;
            else if (k == "--mean-square-displacement-self") msd_self = true;
            else if (k == "-h" || k == "--help") { usage(); return 0; }
            else throw std::runtime_error("option " + k + " is not part of the g(r,t) path");
        }
        if (input.empty() || (nbin == 0 && !(msd || msd_cm || msd_self))) {
            usage();
            return 1;
        }
        if (msd || msd_cm || msd_self) {  // analisi/main.cpp:520-551
            std::cerr << "Mean square displacement calculation ";
            const unsigned f_cm = msd_cm ? 2 : 1;
            if (msd_cm) {
                std::cerr << "of the center of mass and of the atoms is beginning...\n";
            } else {
                std::cerr << " of the atoms is beginning...\n";
                if (msd_self) std::cerr << "In the reference system of each atomic type center of mass...\n";
                else std::cerr << "In the cell coordinate system...\n";
            }
            LammpsFrames fr = read_lammps_binary(input);
            Trajectory tr(fr.positions.data(), fr.velocities.data(), fr.types.data(),
                          fr.boxes.data(), fr.nframes, fr.natoms,
                          fr.triclinic ? BoxFormat::Lammps_triclinic : BoxFormat::Lammps_ortho,
                          false, false);
            using M = MeanSquareDisplacement<Trajectory>;
            BlockAverage<Trajectory, M> avg(&tr, (unsigned)blocks);
            avg.calculate((unsigned)skip, (unsigned)tmax, (unsigned)nthreads, msd_cm, msd_self,
                          dump);
            const unsigned nt = (unsigned)tr.get_ntypes();
            for (unsigned i = 0; i < avg.media()->lunghezza() / nt / f_cm; i++) {
                for (unsigned j = 0; j < nt * f_cm; j++)
                    std::cout << avg.media()->elemento(i * nt * f_cm + j) << " "
                              << avg.varianza()->elemento(i * nt * f_cm + j) << " ";
                std::cout << "\n";
            }
            return 0;
        }
        if (factors.size() != 2)
            throw std::runtime_error("You have to specify the distance range with the option -F.\n");
        std::cerr << "Calculation of g(r,t) -- distinctive and non distinctive part of the van Hove "
                     "function...\n";
        LammpsFrames fr = read_lammps_binary(input);
        // the CLI always wraps (analisi/main.cpp:558)
        Trajectory tr(fr.positions.data(), fr.velocities.data(), fr.types.data(), fr.boxes.data(),
                      fr.nframes, fr.natoms,
                      fr.triclinic ? BoxFormat::Lammps_triclinic : BoxFormat::Lammps_ortho, true,
                      false);
        using G = Gofrt<double, Trajectory>;
        BlockAverage<Trajectory, G> gofr(&tr, (unsigned)blocks);
        gofr.calculate(factors[0], factors[1], nbin, (unsigned)tmax, (unsigned)nthreads,
                       (unsigned)skip, (unsigned)every, dump);
        const unsigned ntyp = (unsigned)(tr.get_ntypes() * (tr.get_ntypes() + 1));
        const unsigned tm = gofr.media()->lunghezza() / nbin / ntyp;
        std::cout << gofr.puntatoreCalcolo()->get_columns_description();
        for (unsigned t = 0; t < tm; t += (unsigned)every) {
            for (unsigned r = 0; r < nbin; r++) {
                std::cout << t << " " << r;
                for (unsigned it = 0; it < ntyp; it++)
                    std::cout << " " << gofr.media()->elemento(t * ntyp * nbin + nbin * it + r) << " "
                              << gofr.varianza()->elemento(t * ntyp * nbin + nbin * it + r);
                std::cout << "\n";
            }
            std::cout << "\n\n";
        }
    } catch (const std::exception &e) {
        std::cerr << e.what() << "\n";
        return 2;
    }
    return 0;
}
