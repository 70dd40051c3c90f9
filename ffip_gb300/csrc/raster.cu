// Material rasterisation on the GPU: the slot tables of the six components
// (slot map, row ranges, g_inf, dt/g_inf, 1/g_inf, pole group, packed
// record, pole amplitudes) built on the device from the geometry list, the
// same tables the host's rasterize_media + Engine::init_media produce.
//
// The rules are the reference's Structure::set_materials_from_geometry with
// No_Average (src/structure.cpp:155-249): the first geometry in list order
// whose strict inside test holds at a grid point decides its medium, else the
// default medium; a point is a slot when its medium differs from the
// default's (another g_inf, or a pole amplitude above 1e-4,
// src/structure.cpp:256-264).  Density boxes interpolate rho trilinearly at
// the point (Two_Medium_Box::get_medium, src/geometry.cpp:68-76) or look the
// medium up along rho (General_Medium_Box, src/geometry.cpp:98-107).  Slots
// are numbered in scan order (z, y, x) of each component's points; pole
// groups (the sets of active pool entries) are numbered per side by first
// appearance, components in order.
//
// Device layout of the work, per component: one thread per point of the
// component's valid box.  Pass 1 marks slot points and counts them per block
// (and records the most active poles of a point); the block offsets are
// scanned on the host; pass 2 evaluates the points again and writes each
// slot at its rank.  A point's pole set is named by a dense key (geometry,
// subset of that geometry's candidate poles); the first slot of each key
// (atomicMin) gives the groups' order once a side's three components are
// done, and pass 3 writes the group numbers and packed records.
//
// The arithmetic of the inside tests and the interpolation is the host's,
// operation for operation, and this file is compiled without contraction
// into fused multiply-adds (as the host code is), so that both give the same
// bits.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.hpp"

namespace ffipg
{
namespace
{
constexpr int kMaxCand = 12;   // candidate poles of one density box on one side
constexpr int kRasterThreads = 256;
constexpr double kPoleTol = 1e-4;

// one geometry as the device sees it, media of one side
struct RGeom
{
    int type;
    double center[3], radius;
    double lo[3], hi[3];
    double p1[3], p2[3];
    int dim[3];
    const double *rho;
    int r0[6][3], r1[6][3];  // index box per component (r0 > r1: empty)
    // BOX / SPHERE: the medium
    double g;
    int nb;
    int pool[kMaxPoles];
    double a[kMaxPoles];
    // density boxes: candidate pool entries (increasing) and their amplitudes
    int ncand;
    int cand[kMaxCand];
    double g1, g2, a1[kMaxCand], a2[kMaxCand];  // TWO_MEDIUM_BOX: medium1, medium2
    int nfun;                                   // GENERAL_MEDIUM_BOX: rho_fun / medium_fun
    const double *rho_fun;                      // [nfun]
    const double *fun_g;                        // [nfun]
    const double *fun_a;                        // [nfun][ncand]
    int key_base;                               // first group key of this geometry
};

struct RasterArgs
{
    int c;                        // component 0..5
    int ng;
    const RGeom *geo;
    int n[3], first[3];           // valid box
    int o[3];                     // doubled-grid origin per axis
    int par[3];                   // component parity per axis
    int64_t Mx_pad, M1;
    double g_def, dt;
    int def_nb;
    int def_pool[kMaxPoles];
    double def_a[kMaxPoles];
    // pass 1
    int *count;                   // per block
    int *maxnb, *err;
    unsigned long long *pole_sum;
    // pass 2
    const int64_t *offset;        // per block
    int64_t nslots;
    int stride;
    int *map;
    int *rows;                    // [row][2]: lo, hi
    void *g, *coef, *inv, *amp;   // field type
    int *key;                     // per slot
    uint8_t *nbs;                 // per slot
    unsigned long long *firstpos; // per key: (c << 40) | slot
    bool fp32;
};

__device__ __forceinline__ int coord_of(const RasterArgs &A, int a, int i)
{
    return A.o[a] + 2 * (i - (a == 0 ? kXFirst : 1)) + A.par[a];
}

// interp_axis of the host (one axis of interpn, include/utility.hpp:670-697)
__device__ int r_interp_axis(double q, int n, int idx[2], double w[2])
{
    if (n == 1)
    {
        idx[0] = 0;
        w[0] = 1;
        return -1;
    }
    if (q <= 0)
    {
        if (q <= -1) return 0;
        idx[0] = 0;
        w[0] = q + 1;
        return 1;
    }
    if (q >= n - 1)
    {
        if (q >= n) return 0;
        idx[0] = n - 1;
        w[0] = (double)n - q;
        return 1;
    }
    size_t i = (size_t)q;
    double tx = q - (double)i;
    idx[0] = (int)i + 1;
    w[0] = tx;
    idx[1] = (int)i;
    w[1] = 1 - tx;
    return 2;
}

__device__ double r_density(const RGeom &G, double x, double y, double z)
{
    double zq = (z - G.p1[2]) / (G.p2[2] - G.p1[2]) * (G.dim[2] - 1);
    double yq = (y - G.p1[1]) / (G.p2[1] - G.p1[1]) * (G.dim[1] - 1);
    double xq = (x - G.p1[0]) / (G.p2[0] - G.p1[0]) * (G.dim[0] - 1);
    int iz[2], iy[2], ix[2];
    double wz[2], wy[2], wx[2];
    const int nz = r_interp_axis(zq, G.dim[2], iz, wz);
    const int ny = r_interp_axis(yq, G.dim[1], iy, wy);
    const int nxt = r_interp_axis(xq, G.dim[0], ix, wx);
    auto at = [&](int k, int j, int i) { return G.rho[((size_t)k * G.dim[1] + j) * G.dim[0] + i]; };
    auto lx = [&](int k, int j) -> double {
        if (nxt == -1) return at(k, j, 0);
        if (nxt == 0) return 0.0;
        if (nxt == 1) return wx[0] * at(k, j, ix[0]);
        return wx[0] * at(k, j, ix[0]) + wx[1] * at(k, j, ix[1]);
    };
    auto ly = [&](int k) -> double {
        if (ny == -1) return lx(k, 0);
        if (ny == 0) return 0.0;
        if (ny == 1) return wy[0] * lx(k, iy[0]);
        return wy[0] * lx(k, iy[0]) + wy[1] * lx(k, iy[1]);
    };
    if (nz == -1) return ly(0);
    if (nz == 0) return 0.0;
    if (nz == 1) return wz[0] * ly(iz[0]);
    return wz[0] * ly(iz[0]) + wz[1] * ly(iz[1]);
}

__device__ __forceinline__ bool r_inside(const RGeom &G, double x, double y, double z)
{
    if (G.type == Geometry::SPHERE)
    {
        double dx = x - G.center[0], dy = y - G.center[1], dz = z - G.center[2];
        return dx * dx + dy * dy + dz * dz < G.radius * G.radius;
    }
    return x > G.lo[0] && x < G.hi[0] && y > G.lo[1] && y < G.hi[1] && z > G.lo[2] && z < G.hi[2];
}

// the medium of one point: g_inf, active poles (pool order) with their
// amplitudes, the group key; returns false when too many poles are active
struct PointMed
{
    double g;
    int nb;
    double a[kMaxPoles];
    int key;
};

// gl / gn: the geometries (in list order) that may contain points of the
// calling block; gl = nullptr: all of them
__device__ bool point_medium(const RasterArgs &A, int i, int j, int k, PointMed &m, const int *gl, int gn)
{
    const double x = coord_of(A, 0, i), y = coord_of(A, 1, j), z = coord_of(A, 2, k);
    const int c = A.c;
    int gi = -1;
    for (int q = 0; q < gn; ++q)
    {
        const int g = gl ? gl[q] : q;
        const RGeom &G = A.geo[g];
        if (i < G.r0[c][0] || i > G.r1[c][0] || j < G.r0[c][1] || j > G.r1[c][1] || k < G.r0[c][2] || k > G.r1[c][2]) continue;
        if (r_inside(G, x, y, z))
        {
            gi = g;
            break;
        }
    }
    if (gi < 0)
    {
        m.g = A.g_def;
        m.nb = A.def_nb;
        for (int q = 0; q < A.def_nb; ++q) m.a[q] = A.def_a[q];
        m.key = 0;
        return true;
    }
    const RGeom &G = A.geo[gi];
    if (G.type == Geometry::BOX || G.type == Geometry::SPHERE)
    {
        m.g = G.g;
        m.nb = G.nb;
        for (int q = 0; q < G.nb; ++q) m.a[q] = G.a[q];
        m.key = G.key_base;
        return true;
    }
    const double v = r_density(G, x, y, z);
    double amp[kMaxCand];
    if (G.type == Geometry::TWO_MEDIUM_BOX)
    {
        // m1 * val + m2 * (1 - val), src/geometry.cpp:75
        m.g = G.g1 * v + G.g2 * (1 - v);
        for (int q = 0; q < G.ncand; ++q) amp[q] = G.a1[q] * v + G.a2[q] * (1 - v);
    }
    else
    {
        // General_Medium_Box: 1-D lookup over rho_fun
        const double q = (v - G.rho_fun[0]) / (G.rho_fun[G.nfun - 1] - G.rho_fun[0]) * (double)(G.nfun - 1);
        int idx[2];
        double w[2];
        const int nt = r_interp_axis(q, G.nfun, idx, w);
        if (nt == -1)
        {
            m.g = G.fun_g[0];
            for (int t = 0; t < G.ncand; ++t) amp[t] = G.fun_a[t];
        }
        else
        {
            m.g = 0;
            for (int t = 0; t < G.ncand; ++t) amp[t] = 0;
            for (int s = 0; s < nt; ++s)
            {
                const double *fa = G.fun_a + (size_t)idx[s] * G.ncand;
                if (s == 0)
                {
                    m.g = w[0] * G.fun_g[idx[0]];
                    for (int t = 0; t < G.ncand; ++t) amp[t] = w[0] * fa[t];
                }
                else
                {
                    m.g = m.g + w[1] * G.fun_g[idx[1]];
                    for (int t = 0; t < G.ncand; ++t) amp[t] = amp[t] + w[1] * fa[t];
                }
            }
        }
    }
    m.nb = 0;
    int mask = 0;
    for (int q = 0; q < G.ncand; ++q)
        if (fabs(amp[q]) > kPoleTol)
        {
            if (m.nb == kMaxPoles) return false;
            m.a[m.nb++] = amp[q];
            mask |= 1 << q;
        }
    m.key = G.key_base + mask;
    return true;
}

__device__ __forceinline__ void point_of(const RasterArgs &A, int64_t t, int &i, int &j, int &k)
{
    i = A.first[0] + (int)(t % A.n[0]);
    j = A.first[1] + (int)(t / A.n[0] % A.n[1]);
    k = A.first[2] + (int)(t / ((int64_t)A.n[0] * A.n[1]));
}

__device__ __forceinline__ bool is_slot(const RasterArgs &A, const PointMed &m) { return !(m.nb == 0 && m.g == A.g_def); }

// The geometries whose index box meets the index box of the block's 256
// points (scan order t0 .. t0 + 255), in list order, into gl (capacity
// kBlockGeoms); returns their count, or -1 when they do not fit (the caller
// then walks the whole list).  Every thread of the block calls it.
constexpr int kBlockGeoms = 256;
__device__ int block_geoms(const RasterArgs &A, int64_t total, int *gl, int *warp_n)
{
    const int64_t t0 = blockIdx.x * (int64_t)kRasterThreads, t1 = min(t0 + kRasterThreads, total) - 1;
    int i0, j0, k0, i1, j1, k1;
    point_of(A, t0, i0, j0, k0);
    point_of(A, t1, i1, j1, k1);
    int lo[3], hi[3];
    lo[2] = k0;
    hi[2] = k1;
    if (k0 == k1 && j0 == j1)
    {
        lo[0] = i0, hi[0] = i1, lo[1] = hi[1] = j0;
    }
    else
    {
        lo[0] = A.first[0], hi[0] = A.first[0] + A.n[0] - 1;
        if (k0 == k1) lo[1] = j0, hi[1] = j1;
        else lo[1] = A.first[1], hi[1] = A.first[1] + A.n[1] - 1;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, c = A.c;
    int n = 0;
    for (int base = 0; base < A.ng; base += kRasterThreads)
    {
        const int g = base + threadIdx.x;
        bool hit = false;
        if (g < A.ng)
        {
            const RGeom &G = A.geo[g];
            hit = true;
            for (int a = 0; a < 3; ++a) hit = hit && G.r0[c][a] <= hi[a] && G.r1[c][a] >= lo[a] && G.r0[c][a] <= G.r1[c][a];
        }
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) warp_n[wid] = __popc(bal);
        __syncthreads();
        int before = 0, all = 0;
        for (int w = 0; w < kRasterThreads / 32; ++w)
        {
            if (w < wid) before += warp_n[w];
            all += warp_n[w];
        }
        if (hit && n + all <= kBlockGeoms) gl[n + before + __popc(bal & ((1u << lane) - 1u))] = g;
        n += all;
        __syncthreads();
        if (n > kBlockGeoms) return -1;
    }
    return n;
}

// pass 1: slot points per block, most active poles, active poles summed
__global__ void __launch_bounds__(kRasterThreads) k_raster_count(const __grid_constant__ RasterArgs A, int64_t total)
{
    __shared__ int gl[kBlockGeoms];
    __shared__ int warp_n[kRasterThreads / 32];
    const int gn = block_geoms(A, total, gl, warp_n);
    const int64_t t = blockIdx.x * (int64_t)kRasterThreads + threadIdx.x;
    bool s = false;
    int nb = 0;
    if (t < total)
    {
        int i, j, k;
        point_of(A, t, i, j, k);
        PointMed m;
        if (!point_medium(A, i, j, k, m, gn < 0 ? nullptr : gl, gn < 0 ? A.ng : gn)) atomicExch(A.err, 1);
        else
        {
            s = is_slot(A, m);
            nb = s ? m.nb : 0;
        }
    }
    const int cnt = __syncthreads_count(s);
    if (nb)
    {
        atomicMax(A.maxnb, nb);
        atomicAdd(A.pole_sum, (unsigned long long)nb);
    }
    if (threadIdx.x == 0) A.count[blockIdx.x] = cnt;
}

template <typename T>
__device__ void write_slot(const RasterArgs &A, int64_t s, const PointMed &m)
{
    T *g = (T *)A.g, *coef = (T *)A.coef, *inv = (T *)A.inv, *amp = (T *)A.amp;
    g[s] = (T)m.g;
    coef[s] = (T)(A.dt / m.g);
    inv[s] = (T)(1 / m.g);
    for (int q = 0; q < m.nb; ++q) amp[(int64_t)q * A.nslots + s] = (T)m.a[q];
}

// pass 2: every slot point at its rank in scan order
__global__ void __launch_bounds__(kRasterThreads) k_raster_emit(const __grid_constant__ RasterArgs A, int64_t total)
{
    __shared__ int warp_tot[kRasterThreads / 32];
    __shared__ int gl[kBlockGeoms];
    const int gn = block_geoms(A, total, gl, warp_tot);
    __syncthreads();
    const int64_t t = blockIdx.x * (int64_t)kRasterThreads + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    bool s = false;
    int i = 0, j = 0, k = 0;
    PointMed m;
    if (t < total)
    {
        point_of(A, t, i, j, k);
        s = point_medium(A, i, j, k, m, gn < 0 ? nullptr : gl, gn < 0 ? A.ng : gn) && is_slot(A, m);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, s);
    if (lane == 0) warp_tot[wid] = __popc(bal);
    __syncthreads();
    int before = 0;
    for (int w = 0; w < wid; ++w) before += warp_tot[w];
    if (!s) return;
    const int64_t slot = A.offset[blockIdx.x] + before + __popc(bal & ((1u << lane) - 1u));
    const int64_t lin = (int64_t)i + A.Mx_pad * ((int64_t)j + A.M1 * k);
    A.map[lin] = (int)slot;
    const int64_t row = (int64_t)j + A.M1 * k;
    atomicMin(&A.rows[2 * row], i);
    atomicMax(&A.rows[2 * row + 1], i);
    if (A.fp32) write_slot<float>(A, slot, m);
    else write_slot<double>(A, slot, m);
    A.key[slot] = m.key;
    A.nbs[slot] = (uint8_t)m.nb;
    atomicMin(&A.firstpos[m.key], ((unsigned long long)A.c << 40) | (unsigned long long)slot);
}

// rows without slots: (1, 0), as the host leaves them
__global__ void k_raster_rows(int *rows, int64_t nrows)
{
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    if (rows[2 * r] > rows[2 * r + 1])
    {
        rows[2 * r] = 1;
        rows[2 * r + 1] = 0;
    }
}

// pass 3: pole group and packed record of every slot
template <typename T>
__global__ void k_raster_groups(const int *key, const uint8_t *nbs, const int *group_of_key, const T *g, const T *coef,
                                const T *inv, uint8_t *group, SlotRec<T> *rec, int64_t n)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int grp = group_of_key[key[s]];
    group[s] = (uint8_t)grp;
    rec[s] = SlotRec<T>{coef[s], inv[s], g[s], (T)(grp + 256 * (int)nbs[s])};
}

void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("rasterisation: ") + what + ": " + cudaGetErrorString(e));
}

// device scratch of one rasterisation, freed on every exit
struct Scratch
{
    std::vector<void *> p;
    ~Scratch()
    {
        for (void *q : p) cudaFree(q);
    }
    template <typename U>
    U *get(size_t n)
    {
        void *q = nullptr;
        ck(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(U)), "cudaMalloc");
        p.push_back(q);
        return (U *)q;
    }
};
} // namespace

void raster_media(const Plan &P, bool fp32, const std::function<void *(size_t)> &alloc, RasterComp out[6],
                  std::vector<PoleGroup> groups[2], cudaStream_t st)
{
    Scratch S;
    const size_t tsz = fp32 ? 4 : 8;
    const int ng = (int)P.geoms.size();
    // the geometries' density arrays, rho_fun and medium_fun tables
    std::vector<RGeom> hg[2];
    for (int side = 0; side < 2; ++side) hg[side].resize(ng);
    // keys: 0 the default medium; then per geometry one key (box, sphere) or
    // one per subset of its candidate poles (density boxes); per key its
    // pool list (resolved lazily from the geometry and the mask)
    std::vector<int> key_geo[2];
    for (int side = 0; side < 2; ++side) key_geo[side].push_back(-1);
    for (int g = 0; g < ng; ++g)
    {
        const Geometry &G = P.geoms[g];
        const double *drho = nullptr;
        if (G.type == Geometry::TWO_MEDIUM_BOX || G.type == Geometry::GENERAL_MEDIUM_BOX)
        {
            double *d = S.get<double>(G.rho.size());
            ck(cudaMemcpyAsync(d, G.rho.data(), G.rho.size() * sizeof(double), cudaMemcpyHostToDevice, st), "cudaMemcpy");
            drho = d;
        }
        for (int side = 0; side < 2; ++side)
        {
            RGeom &R = hg[side][g];
            R = RGeom();
            R.type = (int)G.type;
            for (int a = 0; a < 3; ++a)
            {
                R.center[a] = G.center[a];
                R.lo[a] = G.lo[a];
                R.hi[a] = G.hi[a];
                R.p1[a] = G.p1[a];
                R.p2[a] = G.p2[a];
                R.dim[a] = G.dim[a];
            }
            R.radius = G.radius;
            R.rho = drho;
            for (int c = 0; c < 6; ++c)
                if (!geometry_index_range(P, G, c, R.r0[c], R.r1[c]))
                    for (int a = 0; a < 3; ++a)
                    {
                        R.r0[c][a] = 1;
                        R.r1[c][a] = 0;
                    }
            R.key_base = (int)key_geo[side].size();
            const size_t npool = P.pool[side].size();
            if (G.type == Geometry::BOX || G.type == Geometry::SPHERE)
            {
                R.g = side == 0 ? G.medium.epsilon : G.medium.mu;
                const std::vector<double> &amps = side == 0 ? G.medium.e_amp : G.medium.m_amp;
                R.nb = 0;
                for (size_t q = 0; q < npool && q < amps.size(); ++q)
                    if (std::abs(amps[q]) > kPoleTol)
                    {
                        if (R.nb == kMaxPoles)
                            throw std::runtime_error("a grid point has more than " + std::to_string(kMaxPoles) + " active poles");
                        R.pool[R.nb] = (int)q;
                        R.a[R.nb++] = amps[q];
                    }
                key_geo[side].push_back(g);
                continue;
            }
            // candidate poles: nonzero in either medium (or any medium_fun entry)
            std::vector<const std::vector<double> *> media;
            if (G.type == Geometry::TWO_MEDIUM_BOX)
            {
                media.push_back(side == 0 ? &G.medium1.e_amp : &G.medium1.m_amp);
                media.push_back(side == 0 ? &G.medium2.e_amp : &G.medium2.m_amp);
            }
            else
                for (const PoolMedium &m : G.medium_fun) media.push_back(side == 0 ? &m.e_amp : &m.m_amp);
            std::vector<int> cand;
            for (size_t q = 0; q < npool; ++q)
            {
                bool nz = false;
                for (auto *m : media) nz = nz || (q < m->size() && (*m)[q] != 0.0);
                if (nz) cand.push_back((int)q);
            }
            if ((int)cand.size() > kMaxCand)
                throw RasterUnsupported("device rasterisation: a density box with more than " + std::to_string(kMaxCand) +
                                        " distinct poles");
            R.ncand = (int)cand.size();
            for (int t = 0; t < R.ncand; ++t) R.cand[t] = cand[t];
            auto amp_of = [&](const std::vector<double> &a, int q) { return q < (int)a.size() ? a[q] : 0.0; };
            if (G.type == Geometry::TWO_MEDIUM_BOX)
            {
                R.g1 = side == 0 ? G.medium1.epsilon : G.medium1.mu;
                R.g2 = side == 0 ? G.medium2.epsilon : G.medium2.mu;
                for (int t = 0; t < R.ncand; ++t)
                {
                    R.a1[t] = amp_of(*media[0], cand[t]);
                    R.a2[t] = amp_of(*media[1], cand[t]);
                }
            }
            else
            {
                R.nfun = (int)G.medium_fun.size();
                std::vector<double> fg(R.nfun), fa((size_t)R.nfun * std::max(R.ncand, 1));
                for (int t = 0; t < R.nfun; ++t)
                {
                    fg[t] = side == 0 ? G.medium_fun[t].epsilon : G.medium_fun[t].mu;
                    for (int u = 0; u < R.ncand; ++u) fa[(size_t)t * R.ncand + u] = amp_of(*media[t], cand[u]);
                }
                double *d1 = S.get<double>(G.rho_fun.size()), *d2 = S.get<double>(fg.size()), *d3 = S.get<double>(fa.size());
                ck(cudaMemcpyAsync(d1, G.rho_fun.data(), G.rho_fun.size() * sizeof(double), cudaMemcpyHostToDevice, st), "cudaMemcpy");
                ck(cudaMemcpyAsync(d2, fg.data(), fg.size() * sizeof(double), cudaMemcpyHostToDevice, st), "cudaMemcpy");
                ck(cudaMemcpyAsync(d3, fa.data(), fa.size() * sizeof(double), cudaMemcpyHostToDevice, st), "cudaMemcpy");
                R.rho_fun = d1;
                R.fun_g = d2;
                R.fun_a = d3;
            }
            for (int m = 0; m < (1 << R.ncand); ++m) key_geo[side].push_back(g);
        }
    }
    // the pool list of a key
    auto key_pools = [&](int side, int key) {
        std::vector<int> v;
        const int g = key_geo[side][key];
        if (g < 0)
        {
            const std::vector<double> &amps = side == 0 ? P.default_medium.e_amp : P.default_medium.m_amp;
            for (size_t q = 0; q < P.pool[side].size() && q < amps.size(); ++q)
                if (std::abs(amps[q]) > kPoleTol) v.push_back((int)q);
            return v;
        }
        const RGeom &R = hg[side][g];
        if (R.type == Geometry::BOX || R.type == Geometry::SPHERE) return std::vector<int>(R.pool, R.pool + R.nb);
        const int mask = key - R.key_base;
        for (int t = 0; t < R.ncand; ++t)
            if (mask >> t & 1) v.push_back(R.cand[t]);
        return v;
    };
    int *d_err = S.get<int>(1), *d_maxnb = S.get<int>(1);
    unsigned long long *d_psum = S.get<unsigned long long>(1);
    for (int side = 0; side < 2; ++side)
    {
        groups[side].clear();
        const int nkeys = (int)key_geo[side].size();
        RGeom *d_geo = S.get<RGeom>(ng);
        if (ng) ck(cudaMemcpyAsync(d_geo, hg[side].data(), ng * sizeof(RGeom), cudaMemcpyHostToDevice, st), "cudaMemcpy");
        unsigned long long *d_first = S.get<unsigned long long>(nkeys);
        ck(cudaMemsetAsync(d_first, 0xff, nkeys * sizeof(unsigned long long), st), "cudaMemset");
        // the default medium's own poles
        const std::vector<double> &def_amp = side == 0 ? P.default_medium.e_amp : P.default_medium.m_amp;
        RasterArgs A{};
        A.ng = ng;
        A.geo = d_geo;
        A.g_def = P.g_default[side];
        A.dt = P.dt;
        A.Mx_pad = P.Mx_pad;
        A.M1 = P.M[1];
        for (size_t q = 0; q < P.pool[side].size() && q < def_amp.size(); ++q)
            if (std::abs(def_amp[q]) > kPoleTol)
            {
                if (A.def_nb == kMaxPoles)
                    throw std::runtime_error("a grid point has more than " + std::to_string(kMaxPoles) + " active poles");
                A.def_pool[A.def_nb] = (int)q;
                A.def_a[A.def_nb++] = def_amp[q];
            }
        A.err = d_err;
        A.maxnb = d_maxnb;
        A.pole_sum = d_psum;
        A.firstpos = d_first;
        A.fp32 = fp32;
        std::vector<int *> keys(3, nullptr);
        std::vector<uint8_t *> nbs(3, nullptr);
        for (int c = 3 * side; c < 3 * side + 3; ++c)
        {
            RasterComp &R = out[c];
            R = RasterComp();
            A.c = c;
            int64_t total = 1;
            for (int a = 0; a < 3; ++a)
            {
                A.first[a] = P.vlo[c][a];
                A.n[a] = std::max(0, P.vhi[c][a] - P.vlo[c][a] + 1);
                A.o[a] = P.o[a];
                A.par[a] = comp_parity(c, a);
                total *= A.n[a];
            }
            if (!total) continue;
            const int64_t nblk = (total + kRasterThreads - 1) / kRasterThreads;
            if (nblk > INT_MAX) throw RasterUnsupported("device rasterisation: grid too large");
            int *d_count = S.get<int>(nblk);
            int64_t *d_off = S.get<int64_t>(nblk);
            ck(cudaMemsetAsync(d_err, 0, sizeof(int), st), "cudaMemset");
            ck(cudaMemsetAsync(d_maxnb, 0, sizeof(int), st), "cudaMemset");
            ck(cudaMemsetAsync(d_psum, 0, sizeof(unsigned long long), st), "cudaMemset");
            A.count = d_count;
            k_raster_count<<<(unsigned)nblk, kRasterThreads, 0, st>>>(A, total);
            ck(cudaGetLastError(), "k_raster_count launch");
            std::vector<int> cnt(nblk);
            int herr = 0, hmax = 0;
            unsigned long long hsum = 0;
            ck(cudaMemcpyAsync(cnt.data(), d_count, nblk * sizeof(int), cudaMemcpyDeviceToHost, st), "cudaMemcpy");
            ck(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st), "cudaMemcpy");
            ck(cudaMemcpyAsync(&hmax, d_maxnb, sizeof(int), cudaMemcpyDeviceToHost, st), "cudaMemcpy");
            ck(cudaMemcpyAsync(&hsum, d_psum, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st), "cudaMemcpy");
            ck(cudaStreamSynchronize(st), "cudaStreamSynchronize");
            if (herr) throw std::runtime_error("a grid point has more than " + std::to_string(kMaxPoles) + " active poles");
            std::vector<int64_t> off(nblk);
            int64_t n = 0;
            for (int64_t b = 0; b < nblk; ++b)
            {
                off[b] = n;
                n += cnt[b];
            }
            if (!n) continue;
            if (n > INT_MAX) throw std::runtime_error("too many material slots for one component");
            ck(cudaMemcpyAsync(d_off, off.data(), nblk * sizeof(int64_t), cudaMemcpyHostToDevice, st), "cudaMemcpy");
            R.n = n;
            R.stride = hmax;
            R.pole_sum = (int64_t)hsum;
            const int64_t cells = P.cells(), nrows = (int64_t)P.M[1] * P.M[2];
            R.map = (int *)alloc(cells * sizeof(int));
            R.rows = (RowRange *)alloc(nrows * sizeof(RowRange));
            ck(cudaMemsetAsync(R.map, 0xff, cells * sizeof(int), st), "cudaMemset");
            {
                std::vector<int> init(2 * nrows);
                for (int64_t r = 0; r < nrows; ++r)
                {
                    init[2 * r] = INT_MAX;
                    init[2 * r + 1] = INT_MIN;
                }
                ck(cudaMemcpyAsync(R.rows, init.data(), init.size() * sizeof(int), cudaMemcpyHostToDevice, st), "cudaMemcpy");
                ck(cudaStreamSynchronize(st), "cudaStreamSynchronize");
            }
            R.g = alloc(n * tsz);
            R.coef = alloc(n * tsz);
            R.inv = alloc(n * tsz);
            R.group = (uint8_t *)alloc(n);
            R.rec = alloc(n * 4 * tsz);
            if (hmax)
            {
                R.amp = alloc((size_t)hmax * n * tsz);
                ck(cudaMemsetAsync(R.amp, 0, (size_t)hmax * n * tsz, st), "cudaMemset");
            }
            keys[c - 3 * side] = S.get<int>(n);
            nbs[c - 3 * side] = S.get<uint8_t>(n);
            A.offset = d_off;
            A.nslots = n;
            A.stride = hmax;
            A.map = R.map;
            A.rows = (int *)R.rows;
            A.g = R.g;
            A.coef = R.coef;
            A.inv = R.inv;
            A.amp = R.amp;
            A.key = keys[c - 3 * side];
            A.nbs = nbs[c - 3 * side];
            k_raster_emit<<<(unsigned)nblk, kRasterThreads, 0, st>>>(A, total);
            ck(cudaGetLastError(), "k_raster_emit launch");
            k_raster_rows<<<(unsigned)((nrows + 255) / 256), 256, 0, st>>>((int *)R.rows, nrows);
            ck(cudaGetLastError(), "k_raster_rows launch");
        }
        // pole groups of the side, numbered by first appearance
        std::vector<unsigned long long> first(nkeys);
        ck(cudaMemcpyAsync(first.data(), d_first, nkeys * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st), "cudaMemcpy");
        ck(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        std::map<std::vector<int>, unsigned long long> first_of;
        for (int key = 0; key < nkeys; ++key)
        {
            if (first[key] == ~0ull) continue;
            auto pools = key_pools(side, key);
            auto it = first_of.find(pools);
            if (it == first_of.end() || first[key] < it->second) first_of[pools] = first[key];
        }
        std::vector<std::pair<unsigned long long, std::vector<int>>> order;
        for (auto &kv : first_of) order.emplace_back(kv.second, kv.first);
        std::sort(order.begin(), order.end());
        if (order.size() > 256) throw std::runtime_error("more than 256 distinct pole patterns");
        std::map<std::vector<int>, int> gid;
        for (size_t t = 0; t < order.size(); ++t)
        {
            gid[order[t].second] = (int)t;
            PoleGroup pg;
            pg.pool = order[t].second;
            groups[side].push_back(pg);
        }
        std::vector<int> gok(nkeys, 0);
        for (int key = 0; key < nkeys; ++key)
            if (first[key] != ~0ull) gok[key] = gid[key_pools(side, key)];
        int *d_gok = S.get<int>(nkeys);
        ck(cudaMemcpyAsync(d_gok, gok.data(), nkeys * sizeof(int), cudaMemcpyHostToDevice, st), "cudaMemcpy");
        for (int c = 3 * side; c < 3 * side + 3; ++c)
        {
            RasterComp &R = out[c];
            if (!R.n) continue;
            const unsigned nb = (unsigned)((R.n + 255) / 256);
            if (fp32)
                k_raster_groups<float><<<nb, 256, 0, st>>>(keys[c - 3 * side], nbs[c - 3 * side], d_gok, (const float *)R.g,
                                                          (const float *)R.coef, (const float *)R.inv, R.group,
                                                          (SlotRec<float> *)R.rec, R.n);
            else
                k_raster_groups<double><<<nb, 256, 0, st>>>(keys[c - 3 * side], nbs[c - 3 * side], d_gok, (const double *)R.g,
                                                           (const double *)R.coef, (const double *)R.inv, R.group,
                                                           (SlotRec<double> *)R.rec, R.n);
            ck(cudaGetLastError(), "k_raster_groups launch");
        }
        // the scratch above is freed on return: finish the side's work first
        ck(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    }
}
} // namespace ffipg
