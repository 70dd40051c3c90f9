// Adjoint-gradient kernels: the transpose of trilinear interpolation
// (_ffip.transpose, app/ffip.cpp:308-352; interpn::transpose,
// include/utility.hpp:706-749) and the forward x adjoint correlation of
// Adjoint_Volume.get_sensitivity (ffip/simulation.py:841-869).
#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

namespace ffipg
{
namespace
{
void check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

struct Grid3
{
    double x0, y0, z0, dx, dy, dz;
    int nx, ny, nz;
};

// one axis of interpn::transpose: up to two (index, weight) terms; -1 terms
// means the axis has size 1 and is passed through with weight 1
__device__ __forceinline__ int taxis(double q, int n, int idx[2], double w[2])
{
    if (n == 1) { idx[0] = 0; w[0] = 1.0; return 1; }
    if (q <= 0)
    {
        if (q <= -1) return 0;
        idx[0] = 0; w[0] = 1 + q;
        return 1;
    }
    if (q >= n - 1)
    {
        if (q >= n) return 0;
        idx[0] = n - 1; w[0] = (double)n - q;
        return 1;
    }
    long long i = (long long)q;
    double tx = q - (double)i;
    idx[0] = (int)i + 1; w[0] = tx;
    idx[1] = (int)i; w[1] = 1 - tx;
    return 2;
}

__device__ __forceinline__ void scatter(const Grid3 &g, double x, double y, double z, double val, double *out)
{
    const double sx = (x - g.x0) / g.dx, sy = (y - g.y0) / g.dy, sz = (z - g.z0) / g.dz;
    int iz[2], iy[2], ix[2];
    double wz[2], wy[2], wx[2];
    const int nz = taxis(sz, g.nz, iz, wz), ny = taxis(sy, g.ny, iy, wy), nx = taxis(sx, g.nx, ix, wx);
    for (int a = 0; a < nz; ++a)
    {
        const double va = val * wz[a];
        for (int b = 0; b < ny; ++b)
        {
            const double vb = va * wy[b];
            for (int c = 0; c < nx; ++c)
                atomicAdd(&out[((long long)iz[a] * g.ny + iy[b]) * g.nx + ix[c]], vb * wx[c]);
        }
    }
}

__global__ void k_transpose(Grid3 g, const double *pt, long long n, double *out)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    scatter(g, pt[4 * i], pt[4 * i + 1], pt[4 * i + 2], pt[4 * i + 3], out);
}

__global__ void k_sensitivity(Grid3 g, double wr, double wi, double nr, double ni, const double *fwd, const double *adj,
                              const double *deps, const double *xyz, long long n, double *out)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    // (((w fwd) adj) deps) / norm, left to right as numpy evaluates it
    double br = fwd[2 * i], bi = fwd[2 * i + 1];
    double tr = wr * br - wi * bi, ti = wr * bi + wi * br;            // w * fwd
    br = adj[2 * i]; bi = adj[2 * i + 1];
    double ur = tr * br - ti * bi, ui = tr * bi + ti * br;            // * adj
    br = deps[2 * i]; bi = deps[2 * i + 1];
    tr = ur * br - ui * bi; ti = ur * bi + ui * br;                   // * deps
    // real part of (tr + j ti) / (nr + j ni)
    const double den = nr * nr + ni * ni;
    const double se = (tr * nr + ti * ni) / den;
    scatter(g, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], se, out);
}

Grid3 make_grid(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz)
{
    Grid3 g;
    g.x0 = gx[0]; g.y0 = gy[0]; g.z0 = gz[0];
    g.dx = nx > 1 ? gx[1] - gx[0] : 1;
    g.dy = ny > 1 ? gy[1] - gy[0] : 1;
    g.dz = nz > 1 ? gz[1] - gz[0] : 1;
    g.nx = (int)nx; g.ny = (int)ny; g.nz = (int)nz;
    return g;
}

template <typename F>
int run_scatter(uint64_t nout, double *out, F &&launch)
{
    double *dout = nullptr;
    check(cudaMalloc(&dout, nout * sizeof(double)), "cudaMalloc");
    try
    {
        check(cudaMemset(dout, 0, nout * sizeof(double)), "cudaMemset");
        launch(dout);
        check(cudaGetLastError(), "adjoint kernel launch");
        check(cudaMemcpy(out, dout, nout * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    }
    catch (...)
    {
        cudaFree(dout);
        throw;
    }
    cudaFree(dout);
    return 0;
}

double *to_device(const double *h, uint64_t n, std::vector<double *> &keep)
{
    double *d = nullptr;
    if (!n) return nullptr;
    check(cudaMalloc(&d, n * sizeof(double)), "cudaMalloc");
    keep.push_back(d);
    check(cudaMemcpy(d, h, n * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    return d;
}
} // namespace

int adjoint_transpose(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz,
                      const double *pt, uint64_t npts, double *out)
{
    Grid3 g = make_grid(gx, nx, gy, ny, gz, nz);
    std::vector<double *> keep;
    try
    {
        double *dpt = to_device(pt, 4 * npts, keep);
        run_scatter(nx * ny * nz, out, [&](double *dout) {
            if (npts) k_transpose<<<(unsigned)((npts + 255) / 256), 256>>>(g, dpt, (long long)npts, dout);
        });
    }
    catch (...)
    {
        for (double *p : keep) cudaFree(p);
        throw;
    }
    for (double *p : keep) cudaFree(p);
    return 0;
}

int adjoint_sensitivity(double w_re, double w_im, double norm_re, double norm_im, const double *fwd, const double *adj,
                        const double *deps, const double *xyz, uint64_t n, const double *gx, uint64_t nx,
                        const double *gy, uint64_t ny, const double *gz, uint64_t nz, double *out)
{
    Grid3 g = make_grid(gx, nx, gy, ny, gz, nz);
    std::vector<double *> keep;
    try
    {
        double *df = to_device(fwd, 2 * n, keep), *da = to_device(adj, 2 * n, keep), *de = to_device(deps, 2 * n, keep);
        double *dx = to_device(xyz, 3 * n, keep);
        run_scatter(nx * ny * nz, out, [&](double *dout) {
            if (n) k_sensitivity<<<(unsigned)((n + 255) / 256), 256>>>(g, w_re, w_im, norm_re, norm_im, df, da, de, dx, (long long)n, dout);
        });
    }
    catch (...)
    {
        for (double *p : keep) cudaFree(p);
        throw;
    }
    for (double *p : keep) cudaFree(p);
    return 0;
}

// ffip_transpose_noalloc: the same k_transpose over a fixed, file-scope
// device buffer instead of per-call cudaMalloc/cudaFree.  Layout inside the
// buffer: the 4 * npts point doubles, then the nx * ny * nz output doubles
// (the output region is zeroed on every call; the point region is fully
// overwritten by the copy).  One buffer per device and per process: calls
// that overlap on the same device race on it.
namespace
{
constexpr uint64_t kTransposeScratchDoubles = uint64_t(1) << 20; // 8 MiB
__device__ __align__(256) double g_transpose_scratch[kTransposeScratchDoubles];

// address of g_transpose_scratch on each device, looked up once per device
double *scratch_address(int device)
{
    constexpr int kMaxDevices = 64;
    static double *addr[kMaxDevices] = {};
    if (device < 0 || device >= kMaxDevices) throw std::runtime_error("device ordinal out of range");
    if (!addr[device])
    {
        void *p = nullptr;
        check(cudaGetSymbolAddress(&p, g_transpose_scratch), "cudaGetSymbolAddress");
        addr[device] = static_cast<double *>(p);
    }
    return addr[device];
}
} // namespace

uint64_t adjoint_transpose_noalloc_capacity() { return kTransposeScratchDoubles; }

int adjoint_transpose_noalloc(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz,
                              const double *pt, uint64_t npts, double *out)
{
    const uint64_t nout = nx * ny * nz;
    if (npts > kTransposeScratchDoubles / 4 || nout > kTransposeScratchDoubles - 4 * npts)
        throw std::length_error("ffip_transpose_noalloc: 4 * npts + nx * ny * nz = " + std::to_string(4 * npts + nout) +
                                " doubles exceeds the fixed scratch of " + std::to_string(kTransposeScratchDoubles) +
                                " doubles; use ffip_transpose");
    int device = 0;
    check(cudaGetDevice(&device), "cudaGetDevice");
    double *base = scratch_address(device);
    double *dpt = base, *dout = base + 4 * npts;
    Grid3 g = make_grid(gx, nx, gy, ny, gz, nz);
    if (npts) check(cudaMemcpy(dpt, pt, 4 * npts * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    check(cudaMemset(dout, 0, nout * sizeof(double)), "cudaMemset");
    if (npts) k_transpose<<<(unsigned)((npts + 255) / 256), 256>>>(g, dpt, (long long)npts, dout);
    check(cudaGetLastError(), "adjoint kernel launch");
    check(cudaMemcpy(out, dout, nout * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    return 0;
}
} // namespace ffipg
