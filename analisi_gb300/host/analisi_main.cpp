// `analisi` command line, g(r,t) branch, on the GB300 engine.
//
//   analisi -i traj.bin -g NBIN -F RMIN RMAX [-S TMAX] [-s SKIP] [-e EVERY]
//           [-N THREADS] [-B BLOCKS] [-d]
//
// Same options, defaults and output as the reference's gofr branch
// (analisi/main.cpp:162-232 for the options, :552-584 for the computation and
// the printout): the trajectory is read with pbc wrapping on, split into
// BLOCKS block averages, and each (lag, bin) row prints the mean and variance
// of every channel.  -N is the reference's thread count: the per-thread sums
// it implies are reproduced exactly.  Options of the reference's other
// analyses are rejected.
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "blockaverage.h"
#include "gofrt.h"
#include "lammps_file.h"
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
                 "  -d, --dump-block        append every block's buffer to gofrt.dump\n";
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
    bool dump = false;
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
            else if (k == "-h" || k == "--help") { usage(); return 0; }
            else throw std::runtime_error("option " + k + " is not part of the g(r,t) path");
        }
        if (nbin == 0 || input.empty()) {
            usage();
            return 1;
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
