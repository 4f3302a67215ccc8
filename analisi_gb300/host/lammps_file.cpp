// Binary trajectory reader/writer; the format is described in lammps_file.h.
#include "lammps_file.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <unordered_map>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

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

LammpsMmap::LammpsMmap(const std::string &path)
{
    const int fd = ::open(path.c_str(), O_RDONLY);
    if (fd < 0) throw std::runtime_error("Error opening the trajectory \"" + path + "\"\n");
    struct stat st;
    if (::fstat(fd, &st) != 0) {
        ::close(fd);
        throw std::runtime_error("Error reading the size of \"" + path + "\"");
    }
    size_ = (size_t)st.st_size;
    if (size_ == 0) {
        ::close(fd);
        throw std::runtime_error("empty trajectory file \"" + path + "\"");
    }
    void *m = ::mmap(nullptr, size_, PROT_READ, MAP_PRIVATE, fd, 0);
    ::close(fd);
    if (m == MAP_FAILED) throw std::runtime_error("mmap of \"" + path + "\" failed");
    data_ = static_cast<const char *>(m);
    ::madvise(m, size_, MADV_SEQUENTIAL);
    try {
        // index: every frame's header offset; the first frame's atoms
        Cursor c{data_, data_ + size_};
        while (c.p < c.end) {
            const size_t off = (size_t)(c.p - data_);
            const Header h = read_header(c);
            if (offsets_.empty()) {
                natoms_ = (size_t)h.natoms;
                triclinic_ = h.triclinic != 0;
                types_.assign(natoms_, -1);
                ids_.reserve(natoms_);
            } else if ((size_t)h.natoms != natoms_) {
                std::stringstream ss;
                ss << "Error: at the LAMMPS timestep " << h.timestep
                   << " the number of atoms has changed \n";
                throw std::runtime_error(ss.str());
            }
            const bool first = offsets_.empty();
            offsets_.push_back(off);
            steps_.push_back(h.timestep);
            size_t seen = 0;
            for (int ch = 0; ch < h.nchunk; ++ch) {
                const int nd = c.get<int>();
                if (nd < 0 || nd % 8 != 0)
                    throw std::runtime_error(
                        "Number of bytes of the chunk is not a multiple of the number of atoms\n");
                if (first) {
                    for (int a = 0; a < nd / 8; ++a) {
                        double rec[8];
                        for (int k = 0; k < 8; ++k) rec[k] = c.get<double>();
                        const long long id = std::llround(rec[0]);
                        if (id < 0)
                            throw std::runtime_error("Error: found a negative atomic id in the trajectory");
                        if (seen >= natoms_)
                            throw std::runtime_error("Error: the number of atoms does not correspond to "
                                                     "the sum of the number of atoms of each chunk\n");
                        types_[seen] = (int)std::llround(rec[1]);
                        ids_.push_back(id);
                        ++seen;
                    }
                } else {
                    c.skip((size_t)nd * sizeof(double));
                }
            }
        }
    } catch (...) {
        ::munmap(const_cast<char *>(data_), size_);
        data_ = nullptr;
        throw;
    }
}

LammpsMmap::~LammpsMmap()
{
    if (data_) ::munmap(const_cast<char *>(data_), size_);
}

LammpsFrames LammpsMmap::read(size_t first, size_t count) const
{
    if (first + count > offsets_.size() || first + count < first)
        throw std::runtime_error("requested timestep is out of range");
    LammpsFrames f;
    f.nframes = count;
    f.natoms = natoms_;
    f.triclinic = triclinic_;
    f.types = types_;
    const size_t stride = triclinic_ ? 9 : 6;
    f.positions.assign(count * natoms_ * 3, 0.0);
    f.velocities.assign(count * natoms_ * 3, 0.0);
    f.boxes.assign(count * stride, 0.0);
    // first-frame slot of every id (the reference places later frames' atoms by id)
    std::unordered_map<long long, size_t> slot;
    slot.reserve(natoms_ * 2);
    for (size_t a = 0; a < ids_.size(); ++a) slot.emplace(ids_[a], a);
    for (size_t t = 0; t < count; ++t) {
        Cursor c{data_ + offsets_[first + t], data_ + size_};
        const Header h = read_header(c);
        for (int i = 0; i < 6; ++i) f.boxes[t * stride + i] = h.box[i];
        if (triclinic_)
            for (int i = 0; i < 3; ++i) f.boxes[t * stride + 6 + i] = h.tilt[i];
        f.timesteps.push_back(h.timestep);
        for (int ch = 0; ch < h.nchunk; ++ch) {
            const int nd = c.get<int>();
            for (int a = 0; a < nd / 8; ++a) {
                double rec[8];
                for (int k = 0; k < 8; ++k) rec[k] = c.get<double>();
                auto it = slot.find(std::llround(rec[0]));
                if (it == slot.end()) throw std::runtime_error("Error: unknown atom id in a later frame");
                const size_t idx = it->second;
                for (int k = 0; k < 3; ++k) {
                    f.positions[(t * natoms_ + idx) * 3 + k] = rec[2 + k];
                    f.velocities[(t * natoms_ + idx) * 3 + k] = rec[5 + k];
                }
            }
        }
    }
    return f;
}

LammpsFrames read_lammps_binary(const std::string &path)
{
    const LammpsMmap m(path);
    return m.read(0, m.nframes());
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
