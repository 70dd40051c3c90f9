// run_sim_json: the reference's command-line driver (app/run_sim_json.cpp)
// over the C ABI.  Reads config.json from the working directory (or the path
// given as the first argument), runs the simulation to the config's stop
// condition on the GPU and writes the DFT monitors and geometry-info
// requests.
//
// Datasets.  The reference reads its input datasets from the HDF5 file named
// by "input file" and writes one HDF5 group per output to "fields output
// file" (src/simulation.cpp:151-157, src/dft.cpp:273-320).  This driver links
// no HDF5 library; the same content is exchanged as a directory of .npy files:
// the input datasets are <input file>.d/<dataset name>.npy (float64), and
// every output group is <fields output file>.d/<group name>/ with real.npy,
// imag.npy ([nf][nz][ny][nx]), x.npy, y.npy, z.npy and f.npy, or x/y/z.npy
// for a geometry-info request.  ffip_gb300.runfiles converts both ways with
// h5py where it is installed.
//
// Errors (a bad config, a missing dataset, a CUDA failure) print the message
// and exit with status 1; the reference aborts its MPI job instead.
#include <dirent.h>
#include <sys/stat.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ffip_gb300.h"
#include "json.hpp"

namespace
{
struct Array
{
    std::vector<uint64_t> shape;
    std::vector<double> data;
};

// .npy format version 1.0/2.0, little-endian float64, C order
Array read_npy(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    char magic[6];
    f.read(magic, 6);
    if (!f || std::memcmp(magic, "\x93NUMPY", 6) != 0) throw std::runtime_error(path + ": not a .npy file");
    unsigned char ver[2];
    f.read(reinterpret_cast<char *>(ver), 2);
    uint32_t hlen = 0;
    if (ver[0] == 1)
    {
        unsigned char b[2];
        f.read(reinterpret_cast<char *>(b), 2);
        hlen = b[0] | (b[1] << 8);
    }
    else
    {
        unsigned char b[4];
        f.read(reinterpret_cast<char *>(b), 4);
        hlen = b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)b[3] << 24);
    }
    std::string header(hlen, ' ');
    f.read(&header[0], hlen);
    if (!f) throw std::runtime_error(path + ": truncated header");
    if (header.find("'descr': '<f8'") == std::string::npos && header.find("'descr':'<f8'") == std::string::npos)
        throw std::runtime_error(path + ": only little-endian float64 arrays are read");
    if (header.find("True") != std::string::npos) throw std::runtime_error(path + ": Fortran-ordered arrays are not read");
    Array a;
    const size_t lp = header.find('('), rp = header.find(')');
    if (lp == std::string::npos || rp == std::string::npos) throw std::runtime_error(path + ": no shape");
    std::stringstream ss(header.substr(lp + 1, rp - lp - 1));
    std::string tok;
    uint64_t n = 1;
    while (std::getline(ss, tok, ','))
    {
        size_t b = tok.find_first_not_of(" ");
        if (b == std::string::npos) continue;
        const uint64_t d = std::stoull(tok.substr(b));
        a.shape.push_back(d);
        n *= d;
    }
    a.data.resize(n);
    f.read(reinterpret_cast<char *>(a.data.data()), (std::streamsize)(n * sizeof(double)));
    if (!f) throw std::runtime_error(path + ": truncated data");
    return a;
}

void write_npy(const std::string &path, const std::vector<uint64_t> &shape, const double *data, uint64_t n)
{
    std::string dict = "{'descr': '<f8', 'fortran_order': False, 'shape': (";
    for (size_t i = 0; i < shape.size(); ++i) dict += std::to_string(shape[i]) + (shape.size() == 1 || i + 1 < shape.size() ? ", " : "");
    dict += "), }";
    size_t total = 10 + dict.size() + 1;
    dict += std::string((64 - total % 64) % 64, ' ') + "\n";
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + path);
    const uint16_t hl = (uint16_t)dict.size();
    f.write("\x93NUMPY\x01\x00", 8);
    const char b[2] = {(char)(hl & 0xff), (char)(hl >> 8)};
    f.write(b, 2);
    f.write(dict.data(), (std::streamsize)dict.size());
    f.write(reinterpret_cast<const char *>(data), (std::streamsize)(n * sizeof(double)));
    if (!f) throw std::runtime_error("cannot write " + path);
}

bool is_dir(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

void make_dir(const std::string &p)
{
    if (!is_dir(p) && mkdir(p.c_str(), 0755) != 0) throw std::runtime_error("cannot create directory " + p);
}

void check(int rc, const char *what)
{
    if (rc != FFIP_OK) throw std::runtime_error(std::string(what) + ": " + ffip_last_error());
}
} // namespace

int main(int argc, char **argv)
{
    ffip_sim *sim = nullptr;
    try
    {
        const std::string cfg_path = argc > 1 ? argv[1] : "config.json";
        std::ifstream cf(cfg_path);
        if (!cf) throw std::runtime_error("cannot open " + cfg_path);
        std::stringstream buf;
        buf << cf.rdbuf();
        const std::string text = buf.str();
        const ffipg::Json cfg = ffipg::Json::parse(text);

        // input datasets
        std::vector<std::string> names;
        std::vector<Array> arrays;
        if (cfg.has("input file"))
        {
            const std::string dir = cfg.at("input file").str() + ".d";
            if (is_dir(dir))
            {
                DIR *d = opendir(dir.c_str());
                for (dirent *e = d ? readdir(d) : nullptr; e; e = readdir(d))
                {
                    std::string fn = e->d_name;
                    if (fn.size() > 4 && fn.compare(fn.size() - 4, 4, ".npy") == 0)
                    {
                        names.push_back(fn.substr(0, fn.size() - 4));
                        arrays.push_back(read_npy(dir + "/" + fn));
                    }
                }
                if (d) closedir(d);
            }
        }
        std::vector<ffip_dataset> ds(names.size());
        for (size_t i = 0; i < names.size(); ++i) ds[i] = ffip_dataset{names[i].c_str(), arrays[i].data.data(), arrays[i].data.size()};

        check(ffip_create(text.c_str(), ds.empty() ? nullptr : ds.data(), ds.size(), &sim), "ffip_create");
        check(ffip_run(sim, nullptr), "ffip_run");

        // outputs
        const std::string out_dir = (cfg.has("fields output file") ? cfg.at("fields output file").str() : std::string("output.h5")) + ".d";
        make_dir(out_dir);
        int ngroups = 0;
        check(ffip_output_count(sim, &ngroups), "ffip_output_count");
        for (int g = 0; g < ngroups; ++g)
        {
            char gname[4096];
            check(ffip_output_group(sim, g, gname, sizeof(gname)), "ffip_output_group");
            const std::string gdir = out_dir + "/" + gname;
            make_dir(gdir);
            for (const char *arr : {"real", "imag", "x", "y", "z", "f"})
            {
                uint64_t dims[4];
                int nd = 0;
                int rc = ffip_output_array(sim, g, arr, nullptr, 0, dims, &nd);
                if (rc == FFIP_ERR_NOT_FOUND) continue;
                check(rc, "ffip_output_array");
                std::vector<uint64_t> shape(dims, dims + nd);
                uint64_t n = 1;
                for (uint64_t d : shape) n *= d;
                std::vector<double> v(n);
                check(ffip_output_array(sim, g, arr, v.data(), n, dims, &nd), "ffip_output_array");
                write_npy(gdir + "/" + arr + ".npy", shape, v.data(), n);
            }
        }
        ffip_destroy(sim);
        return 0;
    }
    catch (const std::exception &e)
    {
        std::fprintf(stderr, "run_sim_json: %s\n", e.what());
        if (sim) ffip_destroy(sim);
        return 1;
    }
}
