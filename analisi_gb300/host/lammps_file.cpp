// Binary trajectory reader/writer; the format is described in lammps_file.h.
#include "lammps_file.h"

#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>

namespace analisi_gb300 {

namespace {

struct Cursor {
    const char *p, *end;
    template <typename T>
    T get()
    {
        if (p + sizeof(T) > end) throw std::runtime_error("Error: end of file reached");
        T v;
        std::memcpy(&v, p, sizeof(T));
        p += sizeof(T);
        return v;
    }
    void skip(size_t n)
    {
        if (p + n > end) throw std::runtime_error("Error: end of file reached");
        p += n;
    }
};

struct Header {
    int64_t timestep = 0, natoms = 0;
    int triclinic = 0;
    double box[6] = {0, 0, 0, 0, 0, 0};
    double tilt[3] = {0, 0, 0};
    int nchunk = 0;
};

Header read_header(Cursor &c)
{
    Header h;
    int64_t first = c.get<int64_t>();
    int dpa = 0;
    if (first < 0) {  // LAMMPS 2020 dump header with a magic string
        c.skip((size_t)(-first));
        c.get<int>();                 // endian
        const int revision = c.get<int>();
        h.timestep = c.get<int64_t>();
        h.natoms = c.get<int64_t>();
        h.triclinic = c.get<int>();
        for (int i = 0; i < 6; ++i) c.get<int>();
        for (int i = 0; i < 6; ++i) h.box[i] = c.get<double>();
        if (h.triclinic)
            for (int i = 0; i < 3; ++i) h.tilt[i] = c.get<double>();
        dpa = c.get<int>();
        if (revision > 0x0001) {
            const int ulen = c.get<int>();
            if (ulen > 0) c.skip((size_t)ulen);
            const char time_flag = c.get<char>();
            if (time_flag) c.get<double>();
            const int clen = c.get<int>();
            c.skip((size_t)clen);
        }
        h.nchunk = c.get<int>();
    } else {
        h.timestep = first;
        h.natoms = c.get<int64_t>();
        h.triclinic = c.get<int>();
        for (int i = 0; i < 6; ++i) c.get<int>();
        for (int i = 0; i < 6; ++i) h.box[i] = c.get<double>();
        if (h.triclinic)
            for (int i = 0; i < 3; ++i) h.tilt[i] = c.get<double>();
        dpa = c.get<int>();
        h.nchunk = c.get<int>();
    }
    if (dpa != 8)
        throw std::runtime_error("ERROR: the binary format does not have 8 numbers per atom but it has " +
                                 std::to_string(dpa));
    if (h.nchunk <= 0)
        throw std::runtime_error("Error: the number of chunks of the timestep cannot be <= 0");
    return h;
}

}  // namespace

LammpsFrames read_lammps_binary(const std::string &path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("Error opening the trajectory \"" + path + "\"\n");
    std::vector<char> buf((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    Cursor c{buf.data(), buf.data() + buf.size()};
    LammpsFrames f;
    std::map<long long, size_t> id_index;
    while (c.p < c.end) {
        const Header h = read_header(c);
        if (f.nframes == 0) {
            f.natoms = (size_t)h.natoms;
            f.triclinic = h.triclinic != 0;
            f.types.assign(f.natoms, -1);
        } else if ((size_t)h.natoms != f.natoms) {
            std::stringstream ss;
            ss << "Error: at the LAMMPS timestep " << h.timestep
               << " the number of atoms has changed \n";
            throw std::runtime_error(ss.str());
        }
        const size_t stride = f.triclinic ? 9 : 6;
        const size_t t = f.nframes;
        f.positions.resize((t + 1) * f.natoms * 3);
        f.velocities.resize((t + 1) * f.natoms * 3);
        f.boxes.resize((t + 1) * stride);
        for (int i = 0; i < 6; ++i) f.boxes[t * stride + i] = h.box[i];
        if (f.triclinic)
            for (int i = 0; i < 3; ++i) f.boxes[t * stride + 6 + i] = h.tilt[i];
        f.timesteps.push_back(h.timestep);
        size_t seen = 0;
        for (int ch = 0; ch < h.nchunk; ++ch) {
            const int nd = c.get<int>();
            if (nd % 8 != 0)
                throw std::runtime_error(
                    "Number of bytes of the chunk is not a multiple of the number of atoms\n");
            for (int a = 0; a < nd / 8; ++a) {
                double rec[8];
                for (int k = 0; k < 8; ++k) rec[k] = c.get<double>();
                const long long id = std::llround(rec[0]);
                size_t idx;
                if (t == 0) {
                    if (id < 0) throw std::runtime_error("Error: found a negative atomic id in the trajectory");
                    if (seen >= f.natoms)
                        throw std::runtime_error("Error: the number of atoms does not correspond to the "
                                                 "sum of the number of atoms of each chunk\n");
                    auto ins = id_index.emplace(id, seen);
                    idx = ins.first->second;
                    f.types[idx] = (int)std::llround(rec[1]);
                } else {
                    auto it = id_index.find(id);
                    if (it == id_index.end()) throw std::runtime_error("Error: unknown atom id in a later frame");
                    idx = it->second;
                }
                ++seen;
                for (int k = 0; k < 3; ++k) {
                    f.positions[(t * f.natoms + idx) * 3 + k] = rec[2 + k];
                    f.velocities[(t * f.natoms + idx) * 3 + k] = rec[5 + k];
                }
            }
        }
        ++f.nframes;
    }
    if (f.nframes == 0) throw std::runtime_error("empty trajectory file \"" + path + "\"");
    return f;
}

void write_lammps_binary(const std::string &path, const LammpsFrames &f)
{
    std::ofstream out(path, std::ios::binary);
    if (!out) throw std::runtime_error("cannot write \"" + path + "\"");
    const size_t stride = f.triclinic ? 9 : 6;
    for (size_t t = 0; t < f.nframes; ++t) {
        const int64_t ts = t < f.timesteps.size() ? f.timesteps[t] : (int64_t)t;
        const int64_t na = (int64_t)f.natoms;
        const int tri = f.triclinic ? 1 : 0;
        const int bc[6] = {0, 0, 0, 0, 0, 0};
        const int dpa = 8, nchunk = 1;
        out.write((const char *)&ts, 8);
        out.write((const char *)&na, 8);
        out.write((const char *)&tri, 4);
        out.write((const char *)bc, sizeof bc);
        out.write((const char *)&f.boxes[t * stride], 6 * sizeof(double));
        if (tri) out.write((const char *)&f.boxes[t * stride + 6], 3 * sizeof(double));
        out.write((const char *)&dpa, 4);
        out.write((const char *)&nchunk, 4);
        const int nd = (int)(8 * f.natoms);
        out.write((const char *)&nd, 4);
        for (size_t a = 0; a < f.natoms; ++a) {
            double rec[8] = {(double)(a + 1), (double)f.types[a], 0, 0, 0, 0, 0, 0};
            for (int k = 0; k < 3; ++k) {
                rec[2 + k] = f.positions[(t * f.natoms + a) * 3 + k];
                rec[5 + k] = f.velocities.empty() ? 0.0 : f.velocities[(t * f.natoms + a) * 3 + k];
            }
            out.write((const char *)rec, sizeof rec);
        }
    }
}

}  // namespace analisi_gb300
