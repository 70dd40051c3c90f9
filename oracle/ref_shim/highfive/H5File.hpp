// Stand-in for the HighFive (HDF5) calls the reference makes
// (src/simulation.cpp:151-157,221-231,301-306,435-496; src/dft.cpp:288-318).
//
// Test infrastructure only.  HDF5 is not available here, so a "file" named
// F is the directory F + ".d": a group is a sub-directory and a dataset is a
// little-endian float64 .npy file.  Datasets are written through on every
// write() call.  Reads accept float64 or int64 .npy files.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <sys/stat.h>
#include <vector>

namespace HighFive
{
namespace detail
{
inline void mkdir_p(const std::string &path)
{
    std::string cur;
    std::stringstream ss(path);
    std::string part;
    if (!path.empty() && path[0] == '/') cur = "/";
    while (std::getline(ss, part, '/'))
    {
        if (part.empty()) continue;
        cur += part;
        ::mkdir(cur.c_str(), 0755);
        cur += "/";
    }
}

inline void write_npy(const std::string &path, const std::vector<size_t> &dims, const std::vector<double> &data)
{
    std::string shape = "(";
    for (size_t i = 0; i < dims.size(); ++i)
    {
        shape += std::to_string(dims[i]);
        shape += (dims.size() == 1) ? "," : (i + 1 < dims.size() ? ", " : "");
    }
    shape += ")";
    std::string header = "{'descr': '<f8', 'fortran_order': False, 'shape': " + shape + ", }";
    size_t total = 10 + header.size() + 1;
    size_t pad = (64 - total % 64) % 64;
    header.append(pad, ' ');
    header += '\n';
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw std::runtime_error("cannot write " + path);
    const char magic[] = "\x93NUMPY";
    f.write(magic, 6);
    char ver[2] = {1, 0};
    f.write(ver, 2);
    uint16_t hl = (uint16_t)header.size();
    f.write(reinterpret_cast<const char *>(&hl), 2);
    f.write(header.data(), (std::streamsize)header.size());
    f.write(reinterpret_cast<const char *>(data.data()), (std::streamsize)(data.size() * sizeof(double)));
}

inline std::vector<double> read_npy(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("dataset not found: " + path);
    char magic[6];
    f.read(magic, 6);
    char ver[2];
    f.read(ver, 2);
    uint32_t hl = 0;
    if (ver[0] == 1)
    {
        uint16_t h16;
        f.read(reinterpret_cast<char *>(&h16), 2);
        hl = h16;
    }
    else
        f.read(reinterpret_cast<char *>(&hl), 4);
    std::string header(hl, ' ');
    f.read(&header[0], hl);
    size_t lp = header.find('('), rp = header.find(')');
    size_t n = 1;
    std::string sh = header.substr(lp + 1, rp - lp - 1);
    std::stringstream ss(sh);
    std::string tok;
    while (std::getline(ss, tok, ','))
    {
        if (tok.find_first_not_of(' ') == std::string::npos) continue;
        n *= (size_t)std::stoull(tok);
    }
    std::vector<double> out(n);
    if (header.find("'<f8'") != std::string::npos)
        f.read(reinterpret_cast<char *>(out.data()), (std::streamsize)(n * sizeof(double)));
    else if (header.find("'<i8'") != std::string::npos)
    {
        std::vector<int64_t> tmp(n);
        f.read(reinterpret_cast<char *>(tmp.data()), (std::streamsize)(n * sizeof(int64_t)));
        for (size_t i = 0; i < n; ++i) out[i] = (double)tmp[i];
    }
    else
        throw std::runtime_error("unsupported npy dtype in " + path);
    return out;
}
} // namespace detail

struct MPIOFileDriver
{
    MPIOFileDriver(int, int) {}
};

struct DataSpace
{
    std::vector<size_t> dims;
    DataSpace(const std::vector<size_t> &d) : dims(d) {}
    DataSpace(std::initializer_list<size_t> d) : dims(d) {}
};

struct DataSetStore
{
    std::string path;
    std::vector<size_t> dims;
    std::vector<double> data;
    void flush() const { detail::write_npy(path, dims, data); }
};

class Selection
{
public:
    Selection(std::shared_ptr<DataSetStore> s, std::vector<size_t> off, std::vector<size_t> cnt)
        : s_(std::move(s)), off_(std::move(off)), cnt_(std::move(cnt)) {}

    template <typename T>
    void write(const T *src)
    {
        // row-major hyperslab copy
        const size_t nd = s_->dims.size();
        size_t total = 1;
        for (auto c : cnt_) total *= c;
        std::vector<size_t> idx(nd, 0);
        for (size_t n = 0; n < total; ++n)
        {
            size_t lin = 0;
            for (size_t d = 0; d < nd; ++d) lin = lin * s_->dims[d] + off_[d] + idx[d];
            s_->data[lin] = (double)src[n];
            for (size_t d = nd; d-- > 0;)
            {
                if (++idx[d] < cnt_[d]) break;
                idx[d] = 0;
            }
        }
        s_->flush();
    }
    template <typename T>
    void write(const std::vector<T> &v) { write(v.data()); }

private:
    std::shared_ptr<DataSetStore> s_;
    std::vector<size_t> off_, cnt_;
};

class DataSet
{
public:
    DataSet() = default;
    explicit DataSet(std::shared_ptr<DataSetStore> s) : s_(std::move(s)) {}

    Selection select(const std::vector<size_t> &off, const std::vector<size_t> &cnt) const { return Selection(s_, off, cnt); }

    template <typename T>
    void write(const T *src)
    {
        for (size_t i = 0; i < s_->data.size(); ++i) s_->data[i] = (double)src[i];
        s_->flush();
    }
    template <typename T>
    void write(const std::vector<T> &v) { write(v.data()); }

    void read(std::vector<double> &out) const { out = detail::read_npy(s_->path); }

private:
    std::shared_ptr<DataSetStore> s_;
};

class Group
{
public:
    explicit Group(std::string dir) : dir_(std::move(dir)) { detail::mkdir_p(dir_); }

    template <typename T>
    DataSet createDataSet(const std::string &name, const DataSpace &space)
    {
        auto s = std::make_shared<DataSetStore>();
        s->path = dir_ + "/" + name + ".npy";
        s->dims = space.dims;
        size_t n = 1;
        for (auto d : space.dims) n *= d;
        s->data.assign(n, 0.0);
        s->flush();
        return DataSet(s);
    }

    Group createGroup(const std::string &name) { return Group(dir_ + "/" + name); }

    DataSet getDataSet(const std::string &name) const
    {
        auto s = std::make_shared<DataSetStore>();
        s->path = dir_ + "/" + name + ".npy";
        return DataSet(s);
    }

protected:
    std::string dir_;
};

class File : public Group
{
public:
    enum : unsigned { ReadOnly = 1u, ReadWrite = 2u, Truncate = 4u, Excl = 8u, Debug = 16u, Create = 32u };
    File(const std::string &name, unsigned = ReadOnly, const MPIOFileDriver & = MPIOFileDriver(0, 0)) : Group(name + ".d") {}
};
} // namespace HighFive
