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

// address of g_transpose_scratch on the current device, looked up on every
// call: a host-side lookup that follows the module wherever the current
// context loaded it (a cached address would outlive a cudaDeviceReset), and
// no state is shared between calling threads
double *scratch_address()
{
    void *p = nullptr;
    check(cudaGetSymbolAddress(&p, g_transpose_scratch), "cudaGetSymbolAddress");
    return static_cast<double *>(p);
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
    double *base = scratch_address();
    double *dpt = base, *dout = base + 4 * npts;
    Grid3 g = make_grid(gx, nx, gy, ny, gz, nz);
    if (npts) check(cudaMemcpy(dpt, pt, 4 * npts * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    check(cudaMemset(dout, 0, nout * sizeof(double)), "cudaMemset");
    if (npts) k_transpose<<<(unsigned)((npts + 255) / 256), 256>>>(g, dpt, (long long)npts, dout);
    check(cudaGetLastError(), "adjoint kernel launch");
    check(cudaMemcpy(out, dout, nout * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    return 0;
}

// _ffip.check_inside (app/ffip.cpp:353-387): for each query point, whether
// it lies strictly inside a 2-D polygon (CGAL Polygon_2::bounded_side ==
// ON_BOUNDED_SIDE with the Exact_predicates_inexact_constructions_kernel,
// CGAL >= 4.11).  Points on an edge or a vertex are not inside.  The test is
// a crossing count along +x with exact predicates: a point on an edge (exact
// orientation 0 inside the edge's bounding box) is on the boundary; otherwise
// every edge whose end points straddle the point's y (one end above, the other
// not) and passes to the right of it flips the parity.  The orientation sign
// is exact: Shewchuk's orient2d error-bound filter ("Adaptive Precision
// Floating-Point Arithmetic and Fast Robust Geometric Predicates", 1997), and
// where the filter cannot decide, the determinant expanded into six products
// of coordinates, each split exactly by fma, summed into a nonoverlapping
// expansion (grow-expansion) whose largest component gives the sign.  Exact
// as long as no product of two coordinates overflows or falls below 2^-969
// in magnitude (zero is fine).  For a simple polygon, with or without its
// first vertex repeated at the end, this is CGAL's answer; fewer than three
// distinct vertices give no inside points.
namespace
{
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e)
{
    s = __dadd_rn(a, b);
    const double bv = __dsub_rn(s, a);
    const double av = __dsub_rn(s, bv);
    e = __dadd_rn(__dsub_rn(a, av), __dsub_rn(b, bv));
}

// sign of (ax - cx)(by - cy) - (ay - cy)(bx - cx): > 0 when a, b, c turn
// counter-clockwise
__device__ int orient2d_sign(double ax, double ay, double bx, double by, double cx, double cy)
{
    const double detleft = __dmul_rn(__dsub_rn(ax, cx), __dsub_rn(by, cy));
    const double detright = __dmul_rn(__dsub_rn(ay, cy), __dsub_rn(bx, cx));
    const double det = __dsub_rn(detleft, detright);
    double detsum;
    if (detleft > 0)
    {
        if (detright <= 0) return (det > 0) - (det < 0);
        detsum = __dadd_rn(detleft, detright);
    }
    else if (detleft < 0)
    {
        if (detright >= 0) return (det > 0) - (det < 0);
        detsum = __dsub_rn(-detleft, detright);
    }
    else
        return (det > 0) - (det < 0);
    // (3 + 16 eps) eps, eps = 2^-53
    const double bound = __dmul_rn((3.0 + 16.0 * 0x1p-53) * 0x1p-53, detsum);
    if (det >= bound || -det >= bound) return (det > 0) - (det < 0);
    // exact: ax by - ax cy - cx by - ay bx + ay cx + cy bx (the cx cy terms
    // cancel); each product is hi + lo exactly
    const double fa[6] = {ax, -ax, -cx, -ay, ay, cy};
    const double fb[6] = {by, cy, by, bx, cx, bx};
    double h[12];
#pragma unroll
    for (int t = 0; t < 12; ++t)
    {
        const double p = __dmul_rn(fa[t / 2], fb[t / 2]);
        double q = (t & 1) ? fma(fa[t / 2], fb[t / 2], -p) : p;
        // grow the expansion h[0 .. t-1] by q
#pragma unroll
        for (int i = 0; i < t; ++i)
        {
            double s, e;
            two_sum(q, h[i], s, e);
            h[i] = e;
            q = s;
        }
        h[t] = q;
    }
#pragma unroll
    for (int i = 11; i >= 0; --i)
        if (h[i] != 0) return h[i] > 0 ? 1 : -1;
    return 0;
}

constexpr int kPolyChunk = 2048;  // polygon vertices staged in shared memory per pass

__global__ void __launch_bounds__(256) k_check_inside(const double2 *req, long long n, const double2 *poly, long long m,
                                                      unsigned char *out)
{
    __shared__ double2 v[kPolyChunk + 1];
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = t < n;
    const double2 q = live ? req[t] : make_double2(0, 0);
    bool inside = false, boundary = false;
    for (long long c0 = 0; c0 < m; c0 += kPolyChunk)
    {
        const int len = (int)min((long long)kPolyChunk, m - c0);
        __syncthreads();
        for (int i = threadIdx.x; i <= len; i += blockDim.x) v[i] = poly[(c0 + i) % m];
        __syncthreads();
        if (!live || boundary) continue;
        for (int i = 0; i < len; ++i)
        {
            const double2 a = v[i], b = v[i + 1];
            const bool straddle = (a.y > q.y) != (b.y > q.y);
            const bool in_box = fmin(a.x, b.x) <= q.x && q.x <= fmax(a.x, b.x) && fmin(a.y, b.y) <= q.y && q.y <= fmax(a.y, b.y);
            if (!straddle && !in_box) continue;
            const int o = orient2d_sign(a.x, a.y, b.x, b.y, q.x, q.y);
            if (o == 0 && in_box)
            {
                boundary = true;
                break;
            }
            // the edge crosses y = q.y to the right of q: q is left of the
            // edge directed upwards
            if (straddle && (b.y > a.y ? o > 0 : o < 0)) inside = !inside;
        }
    }
    if (live) out[t] = (inside && !boundary) ? 1 : 0;
}
} // namespace

int check_inside(const double *req, uint64_t n, const double *poly, uint64_t m, unsigned char *out)
{
    if (!n) return 0;
    std::vector<double *> keep;
    unsigned char *dout = nullptr;
    try
    {
        double *dq = to_device(req, 2 * n, keep), *dp = to_device(poly, 2 * m, keep);
        check(cudaMalloc(&dout, n), "cudaMalloc");
        k_check_inside<<<(unsigned)((n + 255) / 256), 256>>>(reinterpret_cast<const double2 *>(dq), (long long)n,
                                                              reinterpret_cast<const double2 *>(dp), (long long)m, dout);
        check(cudaGetLastError(), "k_check_inside launch");
        check(cudaMemcpy(out, dout, n, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    }
    catch (...)
    {
        cudaFree(dout);
        for (double *p : keep) cudaFree(p);
        throw;
    }
    cudaFree(dout);
    for (double *p : keep) cudaFree(p);
    return 0;
}

// Density filters of the design layer (_ffip.TO_convolve / _transpose,
// app/ffip.cpp:222-306): a weighted average over the in-bounds part of an
// odd filter window, and its transpose.  The filter is indexed with the
// first half-width on both axes, as the reference does
// (p2(m - i + r0, n - j + r0)); for square filters that is the usual index.
namespace
{
__device__ __forceinline__ void to_window(int i, int j, int n0, int n1, int r0, int r1, int &l0, int &l1, int &u0, int &u1)
{
    l0 = max(i - r0, 0);
    l1 = max(j - r1, 0);
    u0 = min(i + r0 + 1, n0);
    u1 = min(j + r1 + 1, n1);
}

__global__ void k_to_convolve(const double *in1, int n0, int n1, const double *in2, int m1, int r0, int r1, double *out)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)n0 * n1) return;
    const int i = (int)(t / n1), j = (int)(t % n1);
    int l0, l1, u0, u1;
    to_window(i, j, n0, n1, r0, r1, l0, l1, u0, u1);
    double w = 0, s = 0;
    for (int m = l0; m < u0; ++m)
        for (int n = l1; n < u1; ++n)
        {
            const double f = in2[(int64_t)(m - i + r0) * m1 + (n - j + r0)];
            w += f;
            s += in1[(int64_t)m * n1 + n] * f;
        }
    out[t] = s / w;
}

// transpose, gather form: out(m, n) = sum over (i, j) whose window holds
// (m, n) of in1(i, j) f(m - i + r0, n - j + r0) / w(i, j)
__global__ void k_to_convolve_t(const double *in1, int n0, int n1, const double *in2, int m1, int r0, int r1, double *out)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)n0 * n1) return;
    const int m = (int)(t / n1), n = (int)(t % n1);
    double s = 0;
    for (int i = max(m - r0, 0); i < min(m + r0 + 1, n0); ++i)
        for (int j = max(n - r1, 0); j < min(n + r1 + 1, n1); ++j)
        {
            int l0, l1, u0, u1;
            to_window(i, j, n0, n1, r0, r1, l0, l1, u0, u1);
            double w = 0;
            for (int a = l0; a < u0; ++a)
                for (int b = l1; b < u1; ++b) w += in2[(int64_t)(a - i + r0) * m1 + (b - j + r0)];
            s += in1[(int64_t)i * n1 + j] * in2[(int64_t)(m - i + r0) * m1 + (n - j + r0)] / w;
        }
    out[t] = s;
}
} // namespace

int to_convolve(const double *in1, int n0, int n1, const double *in2, int m0, int m1, double *out, int transpose)
{
    if (n0 < 0 || n1 < 0 || m0 < 1 || m1 < 1) throw std::invalid_argument("bad array shape");
    if (m0 % 2 == 0 || m1 % 2 == 0) throw std::invalid_argument("filter shape is not odd");
    const int r0 = m0 / 2, r1 = m1 / 2;
    // the reference indexes both filter axes with the first half-width
    // (app/ffip.cpp:255): only equal half-widths stay inside the filter
    if (r0 != r1) throw std::invalid_argument("filters with different half-widths are not supported");
    const int64_t n = (int64_t)n0 * n1;
    if (!n) return 0;
    std::vector<double *> keep;
    try
    {
        double *d1 = to_device(in1, n, keep), *d2 = to_device(in2, (uint64_t)m0 * m1, keep);
        double *dout = nullptr;
        check(cudaMalloc(&dout, n * sizeof(double)), "cudaMalloc");
        keep.push_back(dout);
        if (transpose) k_to_convolve_t<<<(unsigned)((n + 255) / 256), 256>>>(d1, n0, n1, d2, m1, r0, r1, dout);
        else k_to_convolve<<<(unsigned)((n + 255) / 256), 256>>>(d1, n0, n1, d2, m1, r0, r1, dout);
        check(cudaGetLastError(), "to_convolve launch");
        check(cudaMemcpy(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    }
    catch (...)
    {
        for (double *p : keep) cudaFree(p);
        throw;
    }
    for (double *p : keep) cudaFree(p);
    return 0;
}
} // namespace ffipg
