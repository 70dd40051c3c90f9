// CUDA kernels (sm_103a) and the CUDA backend of the engine.
//
//   k_update   one half step (H or E) of all three components of a side:
//              curl + CPML psi + constitutive/ADE update + DFT accumulation,
//              threads over (x, y), each marching a chunk of z planes.
//   k_sources  Gaussian dipoles, one thread per distinct source point.
//   k_ghosts   PEC/PMC/periodic ghost planes.
//   k_probe / k_dft_norm   per-step reductions for the stop conditions.
//   k_fused    (fused.cuh) the H and E half steps of one time step in one
//              z-marching pass over the grid.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>
#include <map>
#include <memory>
#include <mutex>
#include <type_traits>
#include <stdexcept>
#include <string>
#include <tuple>

#include "engine.hpp"
#include "fused.cuh"

namespace ffipg
{
// The device rasterisation of the media (raster.cu), on stream st; returns
// with the stream drained
void raster_media(const Plan &p, bool fp32, const std::function<void *(size_t)> &alloc, RasterComp out[6],
                  std::vector<PoleGroup> groups[2], cudaStream_t st);
} // namespace ffipg

// the fused pass's CTA jobs heaviest first (DFT sums, material slots)
#ifndef FFIP_FUSED_HEAVY_FIRST
#define FFIP_FUSED_HEAVY_FIRST 1
#endif
// jobs that meet DFT monitors split along z (1 + frequencies / this many
// pieces; 0: not split)
#ifndef FFIP_FUSED_DFT_SPLIT
#define FFIP_FUSED_DFT_SPLIT 4
#endif
// CPML jobs ordered by the number of axes along which they meet CPML (after
// the DFT and slot weights)
#ifndef FFIP_FUSED_CPML_ORDER
#define FFIP_FUSED_CPML_ORDER 0
#endif
// tile columns with material slots (and no DFT unit) go to the CPML instance
// (off: measured 6 % slower on the 256^3 dispersive workload, where the CPML
// instance is the longer of the two)
#ifndef FFIP_FUSED_SLOTS_TO_P
#define FFIP_FUSED_SLOTS_TO_P 0
#endif

namespace ffipg
{
namespace
{
void check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

constexpr int kUpdTX = 32, kUpdTY = 8, kUpdKZ = 16;

template <typename T, bool IS_E>
__global__ void __launch_bounds__(kUpdTX *kUpdTY) k_update(const __grid_constant__ SideParams<T> p)
{
    const int i = blockIdx.x * kUpdTX + threadIdx.x;
    const int j = blockIdx.y * kUpdTY + threadIdx.y;
    if (i >= p.Mx || j >= p.My) return;
    const int k0 = blockIdx.z * kUpdKZ;
    const int k1 = min(k0 + kUpdKZ, p.Mz);
    constexpr int B = IS_E ? 0 : 3;
    const bool x0ok = i >= p.vlo[0][0] && i <= p.vhi[0][0] && j >= p.vlo[0][1] && j <= p.vhi[0][1];
    const bool x1ok = i >= p.vlo[1][0] && i <= p.vhi[1][0] && j >= p.vlo[1][1] && j <= p.vhi[1][1];
    const bool x2ok = i >= p.vlo[2][0] && i <= p.vhi[2][0] && j >= p.vlo[2][1] && j <= p.vhi[2][1];
    for (int k = k0; k < k1; ++k)
    {
        if (x0ok && k >= p.vlo[0][2] && k <= p.vhi[0][2]) update_point<T, B + 0>(p, i, j, k);
        if (x1ok && k >= p.vlo[1][2] && k <= p.vhi[1][2]) update_point<T, B + 1>(p, i, j, k);
        if (x2ok && k >= p.vlo[2][2] && k <= p.vhi[2][2]) update_point<T, B + 2>(p, i, j, k);
    }
}

template <typename T>
__global__ void k_sources(const __grid_constant__ SourceParams<T> p)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < p.npts) source_point<T>(p, q);
}

template <typename T>
__global__ void k_ghosts(const __grid_constant__ GhostParams<T> p)
{
    ghost_point<T>(p, blockIdx.z, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}

template <typename T>
__global__ void k_probe(const T *f, const int64_t *lin, const double *w, int n, double *out)
{
    // Yee3::interp summation order, include/utility.hpp:997-1002
    double r = 0;
    for (int q = 0; q < n; ++q) r += (double)f[lin[q]] * w[q];
    *out = r;
}

__global__ void k_dft_norm(const double *re, const double *im, int64_t n, double *out)
{
    // deterministic: fixed per-thread strides, fixed tree
    __shared__ double s[256];
    double a = 0;
    for (int64_t i = threadIdx.x; i < n; i += 256) a += re[i] * re[i] + im[i] * im[i];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1)
    {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

// Divergence check: any NaN or infinity among the first n values of nf
// arrays -> *flag = 1 (vector loads; n is a multiple of the 32-element row)
template <typename T>
struct NonfiniteArgs
{
    const T *f[6];
    int nf;
    int64_t n;
};
template <typename T>
__global__ void __launch_bounds__(256) k_nonfinite(const __grid_constant__ NonfiniteArgs<T> a, int *flag)
{
    using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    constexpr int W = sizeof(V) / sizeof(T);
    const int64_t nv = a.n / W;
    bool bad = false;
    for (int i = 0; i < a.nf; ++i)
    {
        const V *p = reinterpret_cast<const V *>(a.f[i]);
        for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nv; t += (int64_t)gridDim.x * blockDim.x)
        {
            const V v = __ldcs(p + t);
            if constexpr (W == 4) bad = bad || !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z) || !isfinite(v.w);
            else bad = bad || !isfinite(v.x) || !isfinite(v.y);
        }
        for (int64_t t = nv * W + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < a.n; t += (int64_t)gridDim.x * blockDim.x)
            bad = bad || !isfinite(a.f[i][t]);
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

// flux through a flux region: per block, partial sums per frequency of
// flux_point over a grid-stride range of integration points (a fixed
// assignment, so the result does not depend on scheduling), then one block
// adds the partials in block order
constexpr int kFluxBlocks = 512;
__global__ void __launch_bounds__(256) k_flux_partial(const __grid_constant__ FluxArgs A, double *partial)
{
    __shared__ double red[256];
    const int64_t np = (int64_t)A.n[0] * A.n[1] * A.n[2];
    for (int f = 0; f < A.nf; ++f)
    {
        double s = 0;
        for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < np; t += (int64_t)gridDim.x * blockDim.x)
            s += flux_point(A, t, f);
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = 128; w > 0; w >>= 1)
        {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[(int64_t)f * gridDim.x + blockIdx.x] = red[0];
        __syncthreads();
    }
}
__global__ void k_flux_total(const double *partial, int nblocks, int nf, double *out)
{
    const int f = threadIdx.x;
    if (f >= nf) return;
    double s = 0;
    for (int b = 0; b < nblocks; ++b) s += partial[(int64_t)f * nblocks + b];
    out[f] = s;
}

// one flag per device and field type: the fused kernels' attributes
// (dynamic shared memory, carveout) are set once on each device
template <typename T>
std::once_flag &fused_attr_once(int dev)
{
    static std::mutex m;
    static std::map<int, std::unique_ptr<std::once_flag>> flags;
    std::lock_guard<std::mutex> g(m);
    auto &f = flags[dev];
    if (!f) f.reset(new std::once_flag);
    return *f;
}

// cuTensorMapEncodeTiled from the driver, without linking libcuda
PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    // looked up once per process (a function-local static is initialised by
    // one thread; a throw leaves it to the next call)
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        check(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q),
              "cudaGetDriverEntryPoint(cuTensorMapEncodeTiled)");
        if (q != cudaDriverEntryPointSuccess || !p) throw std::runtime_error("cuTensorMapEncodeTiled not available");
        return (PFN_cuTensorMapEncodeTiled_v12000)p;
    }();
    return fn;
}

// shared-memory carveout of the fused pass in percent of the maximum; -1:
// sized from the instances' shared memory (tuning builds may override it)
#ifndef FFIP_FUSED_CARVEOUT
#define FFIP_FUSED_CARVEOUT -1
#endif

// 3-D tiled map over one (Mx_pad, My, Mz) field array with a box of
// (bx, by, 1) elements; out-of-range boxes fill zeros.
template <typename T>
CUtensorMap make_map(const T *base, int Mx, int My, int Mz, int bx, int by)
{
    CUtensorMap m;
    cuuint64_t dims[3] = {(cuuint64_t)Mx, (cuuint64_t)My, (cuuint64_t)Mz};
    cuuint64_t strides[2] = {(cuuint64_t)Mx * sizeof(T), (cuuint64_t)Mx * My * sizeof(T)};
    cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = encode_fn()(&m, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                             const_cast<T *>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

class CudaBackend : public Backend
{
public:
    explicit CudaBackend(int device)
    {
        int n = 0;
        check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (n < 1) throw std::runtime_error("no CUDA device");
        if (device < 0) check(cudaGetDevice(&device), "cudaGetDevice");
        if (device >= n) throw std::runtime_error("CUDA device index out of range");
        dev_ = device;
        check(cudaSetDevice(dev_), "cudaSetDevice");
        check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    }
    ~CudaBackend() override
    {
        cudaSetDevice(dev_);
        cudaStreamSynchronize(stream_);
        if (err_) cudaFree(err_);
        if (flag_) cudaFree(flag_);
        for (auto &kv : jobs_) cudaFree(kv.second.dev);
        if (side_) cudaStreamDestroy(side_);
        if (fork_) cudaEventDestroy(fork_);
        if (join_) cudaEventDestroy(join_);
        if (face_h_) cudaEventDestroy(face_h_);
        for (auto &ev : pass_ev_)
        {
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
        cudaStreamDestroy(stream_);
    }
    // every entry re-selects the handle's device: calls may come from any thread
    void use() const { check(cudaSetDevice(dev_), "cudaSetDevice"); }
    void *alloc(size_t bytes) override
    {
        use();
        void *p = nullptr;
        check(cudaMalloc(&p, bytes), "cudaMalloc");
        check(cudaMemsetAsync(p, 0, bytes, stream_), "cudaMemsetAsync");
        return p;
    }
    void release(void *p) override
    {
        cudaSetDevice(dev_);
        cudaStreamSynchronize(stream_);
        cudaFree(p);
    }
    void h2d(void *dst, const void *src, size_t bytes) override
    {
        use();
        h2d_bytes += bytes;
        check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream_), "cudaMemcpy H2D");
        check(cudaStreamSynchronize(stream_), "h2d sync");
    }
    void d2h(void *dst, const void *src, size_t bytes) override
    {
        use();
        d2h_bytes += bytes;
        check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream_), "cudaMemcpy D2H");
        check(cudaStreamSynchronize(stream_), "d2h sync");
    }
    void zero(void *p, size_t bytes) override
    {
        use();
        check(cudaMemsetAsync(p, 0, bytes, stream_), "cudaMemsetAsync");
    }
    void sync() override
    {
        use();
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
        check_err();
    }

    template <typename T>
    void update_t(const SideParams<T> &p, bool is_e)
    {
        use();
        dim3 block(kUpdTX, kUpdTY);
        dim3 grid((p.Mx + kUpdTX - 1) / kUpdTX, (p.My + kUpdTY - 1) / kUpdTY, (p.Mz + kUpdKZ - 1) / kUpdKZ);
        if (is_e) k_update<T, true><<<grid, block, 0, stream_>>>(p);
        else k_update<T, false><<<grid, block, 0, stream_>>>(p);
        check(cudaGetLastError(), "k_update launch");
    }
    void update(const SideParams<double> &p, bool is_e) override { update_t(p, is_e); }
    void update(const SideParams<float> &p, bool is_e) override { update_t(p, is_e); }

    bool has_fused() const override { return true; }

    template <typename T>
    int fused_t(const FusedParams<T> &p, const GhostParams<T> *hg)
    {
        use();
        // interior instance (SH: its tiles define the column grid) and CPML
        // instance (SP: TX / SP::TX jobs per column)
        using SH = FusedShape<T, false>;
        using SP = FusedShape<T, true>;
        using LY = FusedLayout<T, false>;
        using LP = FusedLayout<T, true>;
        static_assert(SH::TX % SP::TX == 0 && SH::TY == SP::TY && SH::KCH == SP::KCH, "instance shapes do not nest");
        if (!err_)
        {
            check(cudaMalloc(&err_, sizeof(int)), "cudaMalloc");
            check(cudaMemsetAsync(err_, 0, sizeof(int), stream_), "cudaMemsetAsync");
        }
        // kernel attributes are per device: set once on each device, by the
        // first handle that launches there, before its first launch (no
        // handle changes them while another one's kernels run)
        std::call_once(fused_attr_once<T>(dev_), [&] {
            // shared memory for the CTAs per SM each instance is built for
            // (plus the 1 KB the system reserves per CTA), the same carveout
            // for both so that they share SMs; the rest of the unified
            // L1/shared array stays L1 (about 60 KB instead of 28 KB in fp32),
            // which the psi staging, the slot loads and the small pole tables
            // go through
            int maxsm = 0;
            check(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev_), "cudaDeviceGetAttribute");
            const int64_t need = std::max<int64_t>((int64_t)SP::MINB * (LP::SMEM_PML + 1024), (int64_t)SH::MINB * (LY::SMEM + 1024));
            const int carve = FFIP_FUSED_CARVEOUT >= 0 ? FFIP_FUSED_CARVEOUT
                                                       : (int)std::min<int64_t>(100, (need * 100 + maxsm - 1) / std::max(maxsm, 1));
            for (int v = 0; v < 4; ++v)
            {
                const int pml = v & 1;
                const auto fn = v == 0 ? k_fused<T, false, false> : v == 1 ? k_fused<T, true, false> : v == 2 ? k_fused<T, false, true>
                                                                                                           : k_fused<T, true, true>;
                check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, pml ? LP::SMEM_PML : LY::SMEM),
                      "cudaFuncSetAttribute");
                check(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, carve), "cudaFuncSetAttribute");
            }
        });
        FusedLaunch<T> L;
        FusedLaunch<T> LC;  // the CPML instance's copy: tensor maps of its box width
        for (int c = 0; c < 3; ++c)
        {
            L.tm_e[c] = map_for(p.ein[c], p.e.Mx, p.e.My, p.e.Mz, SH::BX, SH::TY + 2);
            L.tm_h[c] = map_for(p.hin[c], p.e.Mx, p.e.My, p.e.Mz, SH::BX, SH::TY + 1);
            LC.tm_e[c] = map_for(p.ein[c], p.e.Mx, p.e.My, p.e.Mz, SP::BX, SP::TY + 2);
            LC.tm_h[c] = map_for(p.hin[c], p.e.Mx, p.e.My, p.e.Mz, SP::BX, SP::TY + 1);
        }
        // the DFT sums of the monitored points are added inside the pass
        L.fp = p;
        L.err = err_;
        // valid extents over all six components
        int xend = 0, yend = 0, kbeg = p.e.Mz, kend = 0;
        for (int sd = 0; sd < 2; ++sd)
        {
            const SideParams<T> &P = sd == 0 ? p.e : p.h;
            for (int c = 0; c < 3; ++c)
            {
                xend = std::max(xend, P.vhi[c][0] + 1);
                yend = std::max(yend, P.vhi[c][1] + 1);
                kbeg = std::min(kbeg, P.vlo[c][2]);
                kend = std::max(kend, P.vhi[c][2] + 1);
            }
        }
        // tiles start at the first index holding grid points (kXFirst along
        // x, 1 along y); one or two layers beyond a whole number of tiles go
        // to k_face
        // x is cut into units of the CPML instance's tile width: a unit
        // that touches CPML runs as a CPML job, two (or TX / TX_P) adjacent
        // units without CPML as one interior job
        int nbx, nby;
        fused_limits(xend, yend, kXFirst, SP::TX, SH::TY, nbx, nby, L.xlim, L.ylim);
        L.xend = xend;
        L.yend = yend;
        L.kbeg = kbeg;
        L.kend = std::max(kend, kbeg + 1);
        dim3 block(32, 8);  // 8 warps; each thread owns SH::RPT rows and SH::NPT columns of the tile
        // z chunk length: KCH planes, KCH_SHORT when that gives fewer than 20
        // waves of CTAs, fewer still when the grid has too few tiles to fill
        // the GPU twice (each chunk recomputes one H plane, so at least 4)
        if (!nsm_) check(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev_), "cudaDeviceGetAttribute");
        const int64_t tiles = (int64_t)std::max((nbx * SP::TX + SH::TX - 1) / SH::TX, 1) * std::max(nby, 1);
        const int64_t slots = (int64_t)nsm_ * SH::MINB;  // CTAs resident at once
        const int64_t want = 2 * slots;                  // CTAs for two waves
        const int64_t zlen = L.kend - L.kbeg;
        const int kmax = zlen * tiles < 20 * slots * SH::KCH ? SH::KCH_SHORT : SH::KCH;
        const int kch = (int)std::max<int64_t>(4, std::min<int64_t>(kmax, (zlen * tiles + want - 1) / want));
        const Jobs &J = jobs_for(p, L, nbx, nby, SH::TX, SP::TX, SH::TY, kch);
        LC.fp = L.fp;
        LC.err = L.err;
        LC.xlim = L.xlim;
        LC.ylim = L.ylim;
        LC.xend = L.xend;
        LC.yend = L.yend;
        LC.kbeg = L.kbeg;
        LC.kend = L.kend;
        // E points the pass owns and the PEC / PMC faces it mirrors into
        // the halo of its first tiles (fused_plan.hpp)
        const bool ghost = hg && hg->nfaces > 0;
        const FusedOwnership own = fused_ownership(p.e.vlo, p.e.vhi, ghost ? hg->faces : nullptr, ghost ? hg->nfaces : 0, kXFirst,
                                                   FFIP_FUSED_HALO_MIRROR != 0);
        std::memcpy(L.elo, own.elo, sizeof L.elo);
        std::memcpy(L.ehi, own.ehi, sizeof L.ehi);
        std::memcpy(L.hmirror, own.hmirror, sizeof L.hmirror);
        std::memcpy(L.hghost, own.hghost, sizeof L.hghost);
        std::memcpy(LC.elo, own.elo, sizeof LC.elo);
        std::memcpy(LC.ehi, own.ehi, sizeof LC.ehi);
        std::memcpy(LC.hmirror, own.hmirror, sizeof LC.hmirror);
        std::memcpy(LC.hghost, own.hghost, sizeof LC.hghost);
        // grids with ghost faces take the pass's GH copy (mirrored halo,
        // masked stores of the deferred E points)
        const bool gh = ghost;
        const FaceList fl_h = fused_face_list(p.h.vlo, p.h.vhi, nullptr, nullptr, L.xlim, L.ylim);
        const FaceList fl_e = fused_face_list(p.e.vlo, p.e.vhi, L.elo, L.ehi, L.xlim, L.ylim);
        int n = 0;
        // a second stream runs the interior instance beside the CPML one, and
        // the H half of k_face (it reads only step-n fields) beside both
        const bool fork = (J.ni > 0 && J.nb > 0) || fl_h.total > 0;
        if (fork)
        {
            if (!side_)
            {
                check(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking), "cudaStreamCreate");
                check(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming), "cudaEventCreate");
                check(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming), "cudaEventCreate");
                check(cudaEventCreateWithFlags(&face_h_, cudaEventDisableTiming), "cudaEventCreate");
            }
            check(cudaEventRecord(fork_, stream_), "cudaEventRecord");
            check(cudaStreamWaitEvent(side_, fork_, 0), "cudaStreamWaitEvent");
        }
        cudaEvent_t pass_end = nullptr;
        if (time_pass_)
        {
            // at most kPassEvents pairs: fold the elapsed times of a full pool
            // into the running sum (waits for the passes already issued)
            if (pass_n_ == kPassEvents) pass_acc_ += drain_passes();
            if (pass_n_ == pass_ev_.size())
            {
                cudaEvent_t a, b;
                check(cudaEventCreate(&a), "cudaEventCreate");
                if (cudaEventCreate(&b) != cudaSuccess)
                {
                    cudaEventDestroy(a);
                    throw std::runtime_error("cudaEventCreate failed");
                }
                pass_ev_.emplace_back(a, b);
            }
            check(cudaEventRecord(pass_ev_[pass_n_].first, stream_), "cudaEventRecord");
            pass_end = pass_ev_[pass_n_++].second;
        }
        // the H half of k_face reads only step-n fields: first on the side
        // stream, ahead of the interior instance
        if (fl_h.total > 0)
        {
            k_face<T, false><<<(unsigned)((fl_h.total + 255) / 256), 256, 0, side_>>>(L, fl_h);
            check(cudaGetLastError(), "k_face launch");
            check(cudaEventRecord(face_h_, side_), "cudaEventRecord");
            ++n;
        }
        if (J.nb > 0)
        {
            LC.jobs = J.dev;
            if (gh) k_fused<T, true, true><<<J.nb, block, LP::SMEM_PML, stream_>>>(LC);
            else k_fused<T, true, false><<<J.nb, block, LP::SMEM_PML, stream_>>>(LC);
            check(cudaGetLastError(), "k_fused launch");
            ++n;
        }
        if (J.ni > 0)
        {
            L.jobs = J.dev + J.nb;
            if (gh) k_fused<T, false, true><<<J.ni, block, LY::SMEM, J.nb > 0 ? side_ : stream_>>>(L);
            else k_fused<T, false, false><<<J.ni, block, LY::SMEM, J.nb > 0 ? side_ : stream_>>>(L);
            check(cudaGetLastError(), "k_fused launch");
            ++n;
        }
        // E of the face layers reads the new H of the face layers and of the
        // tiles next to them; when those tiles are all CPML jobs it follows the
        // CPML instance on the main stream, beside the interior instance
        // (not with ghost faces: the E layers next to them wait for the
        // ghost planes, which need every H of the step)
        const unsigned e_blocks = (unsigned)((fl_e.total + 255) / 256);
        const bool early_face = fl_e.total > 0 && J.nb > 0 && J.face_in_pml && !ghost;
        if (early_face)
        {
            if (fl_h.total > 0) check(cudaStreamWaitEvent(stream_, face_h_, 0), "cudaStreamWaitEvent");
            k_face<T, true><<<e_blocks, 256, 0, stream_>>>(L, fl_e);
            check(cudaGetLastError(), "k_face launch");
            ++n;
        }
        if (fork)
        {
            check(cudaEventRecord(join_, side_), "cudaEventRecord");
            check(cudaStreamWaitEvent(stream_, join_, 0), "cudaStreamWaitEvent");
        }
        if (pass_end) check(cudaEventRecord(pass_end, stream_), "cudaEventRecord");
        if (ghost)
        {
            ghosts_t(*hg);
            ++n;
        }
        if (fl_e.total > 0 && !early_face)
        {
            k_face<T, true><<<e_blocks, 256, 0, stream_>>>(L, fl_e);
            check(cudaGetLastError(), "k_face launch");
            ++n;
        }
        return n;
    }
    int fused(const FusedParams<double> &p, const GhostParams<double> *hg) override { return fused_t(p, hg); }
    int fused(const FusedParams<float> &p, const GhostParams<float> *hg) override { return fused_t(p, hg); }

    // CTA jobs of the fused pass (x0, y0, k0, k1): the jobs whose tile, halo
    // and planes touch a CPML point first (nb of them), then the others (ni).
    // Built once per grid, CPML tables and media.  nbx counts x units of
    // TXP columns (the CPML instance's tile width); an interior job covers
    // TX / TXP adjacent units.
    struct Jobs
    {
        int4 *dev{nullptr};
        int nb{0}, ni{0};
        // no job of the instance without CPML code holds the last x tile or
        // the last y tile: the tiles whose new H the E half of k_face reads
        // all belong to the CPML instance
        bool face_in_pml{false};
    };
    template <typename T>
    const Jobs &jobs_for(const FusedParams<T> &p, const FusedLaunch<T> &L, int nbx, int nby, int TX, int TXP, int TY, int KCH)
    {
        const SideParams<T> &P = p.e;
        char key[256];
        std::snprintf(key, sizeof key, "%d %d %d %d %d %d %d %d %d %d %p %d %p %p %p", L.xlim, L.ylim, L.kbeg, L.kend, nbx, nby, TX,
                      TXP, TY, KCH, (const void *)P.pc[0][0], (int)sizeof(T), (const void *)P.slot[0].rows,
                      (const void *)P.slot[1].rows, (const void *)P.slot[2].rows);
        auto it = jobs_.find(key);
        if (it != jobs_.end()) return it->second;
        // the job lists' inputs copied back from the device: CPML flags per
        // position along each axis (either parity), E slot row ranges, DFT
        // unit boxes (fused_plan.hpp builds the lists)
        JobInputs I;
        const int len[3] = {L.xend, P.My, P.Mz};  // table lengths (x: the valid extent, not the padded row)
        for (int a = 0; a < 3; ++a)
        {
            I.pml[a].assign(len[a], 0);
            if (!P.pc[0][0]) continue;
            for (int q = 0; q < 2; ++q)
            {
                std::vector<T> c(len[a]);
                check(cudaMemcpy(c.data(), P.pc[a][q], len[a] * sizeof(T), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
                for (int i = 0; i < len[a]; ++i) I.pml[a][i] |= c[i] != T(0);
            }
        }
        for (int c = 0; c < 3; ++c)
            if (P.slot[c].map)
            {
                I.rows[c].resize((size_t)P.My * P.Mz);
                check(cudaMemcpy(I.rows[c].data(), P.slot[c].rows, I.rows[c].size() * sizeof(RowRange), cudaMemcpyDeviceToHost),
                      "cudaMemcpy D2H");
            }
        for (int sd = 0; sd < 2; ++sd)
        {
            const SideParams<T> &S = sd ? p.h : p.e;
            for (int u = 0; u < S.nunits; ++u)
            {
                DftBox d;
                for (int a = 0; a < 3; ++a)
                {
                    d.i0[a] = S.units[u].i0[a];
                    d.ld[a] = S.units[u].ld[a];
                }
                d.nf = S.units[u].nf;
                I.dft.push_back(d);
            }
        }
        I.My = P.My;
        I.Mz = P.Mz;
        I.xlim = L.xlim;
        I.ylim = L.ylim;
        I.kbeg = L.kbeg;
        I.kend = L.kend;
        I.nbx = nbx;
        I.nby = nby;
        I.TX = TX;
        I.TXP = TXP;
        I.TY = TY;
        I.KCH = KCH;
        const JobLists JL = fused_jobs(I, kXFirst, FFIP_FUSED_SLOTS_TO_P != 0, FFIP_FUSED_DFT_SPLIT, FFIP_FUSED_HEAVY_FIRST != 0,
                                       FFIP_FUSED_CPML_ORDER != 0);
        Jobs J;
        J.nb = (int)JL.b.size();
        J.ni = (int)JL.in.size();
        J.face_in_pml = JL.face_in_pml;
        std::vector<int4> b;
        b.reserve(JL.b.size() + JL.in.size());
        for (const JobBox &jb : JL.b) b.push_back(make_int4(jb.x, jb.y, jb.z, jb.w));
        for (const JobBox &jb : JL.in) b.push_back(make_int4(jb.x, jb.y, jb.z, jb.w));
        // a new media or grid makes a new key (the slot row arrays are new):
        // keep the lists of the last few only (a design loop re-rasterises
        // every iteration); cudaFree waits for the launches that read them
        if (jobs_.size() >= kJobCache)
        {
            auto old = jobs_.find(jobs_order_.front());
            if (old != jobs_.end())
            {
                check(cudaFree(old->second.dev), "cudaFree");
                jobs_.erase(old);
            }
            jobs_order_.erase(jobs_order_.begin());
        }
        check(cudaMalloc(&J.dev, b.size() * sizeof(int4)), "cudaMalloc");
        check(cudaMemcpy(J.dev, b.data(), b.size() * sizeof(int4), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        jobs_order_.push_back(key);
        return jobs_[key] = J;
    }

    template <typename T>
    CUtensorMap map_for(const T *base, int Mx, int My, int Mz, int bx, int by)
    {
        auto key = std::make_tuple((const void *)base, bx, by);
        auto it = maps_.find(key);
        if (it != maps_.end()) return it->second;
        CUtensorMap m = make_map(base, Mx, My, Mz, bx, by);
        maps_[key] = m;
        return m;
    }

    // raises if a bounded wait inside the fused kernel gave up
    void check_err()
    {
        if (!err_) return;
        int e = 0;
        check(cudaMemcpyAsync(&e, err_, sizeof(int), cudaMemcpyDeviceToHost, stream_), "cudaMemcpy err flag");
        check(cudaStreamSynchronize(stream_), "sync");
        if (e)
            throw DeviceTimeout("fused kernel: a wait on its TMA rings or on its CTA's threads timed out; the field "
                                "state is invalid until ffip_reset");
    }
    void flux(const FluxArgs &A0, double *out) override
    {
        use();
        FluxArgs A = A0;
        std::vector<double *> keep;
        auto up = [&](const double *h, size_t n) {
            double *d = nullptr;
            check(cudaMalloc(&d, n * sizeof(double)), "cudaMalloc");
            keep.push_back(d);
            check(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, stream_), "cudaMemcpy H2D");
            return d;
        };
        try
        {
            A.x = up(A0.x, A0.n[0]);
            A.y = up(A0.y, A0.n[1]);
            A.z = up(A0.z, A0.n[2]);
            A.w = up(A0.w, (size_t)A0.n[0] * A0.n[1] * A0.n[2]);
            double *partial = nullptr, *dout = nullptr;
            check(cudaMalloc(&partial, (size_t)kFluxBlocks * A.nf * sizeof(double)), "cudaMalloc");
            keep.push_back(partial);
            check(cudaMalloc(&dout, A.nf * sizeof(double)), "cudaMalloc");
            keep.push_back(dout);
            k_flux_partial<<<kFluxBlocks, 256, 0, stream_>>>(A, partial);
            check(cudaGetLastError(), "k_flux_partial launch");
            k_flux_total<<<1, kMaxFluxFreqs, 0, stream_>>>(partial, kFluxBlocks, A.nf, dout);
            check(cudaGetLastError(), "k_flux_total launch");
            check(cudaMemcpyAsync(out, dout, A.nf * sizeof(double), cudaMemcpyDeviceToHost, stream_), "cudaMemcpy D2H");
            check(cudaStreamSynchronize(stream_), "sync");
            d2h_bytes += A.nf * sizeof(double);
        }
        catch (...)
        {
            cudaStreamSynchronize(stream_);
            for (double *d : keep) cudaFree(d);
            throw;
        }
        for (double *d : keep) cudaFree(d);
    }
    bool can_rasterize() const override { return true; }
    void rasterize(const Plan &plan, bool fp32, const std::function<void *(size_t)> &alloc, RasterComp out[6],
                   std::vector<PoleGroup> groups[2]) override
    {
        use();
        raster_media(plan, fp32, alloc, out, groups, stream_);
    }
    void clear_error() override
    {
        if (!err_) return;
        use();
        check(cudaMemsetAsync(err_, 0, sizeof(int), stream_), "cudaMemsetAsync");
    }

    template <typename T>
    bool any_nonfinite_t(const T *const *f, int nf, int64_t n)
    {
        use();
        if (!flag_) check(cudaMalloc(&flag_, sizeof(int)), "cudaMalloc");
        check(cudaMemsetAsync(flag_, 0, sizeof(int), stream_), "cudaMemsetAsync");
        if (!nsm_) check(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev_), "cudaDeviceGetAttribute");
        NonfiniteArgs<T> a{};
        for (int i = 0; i < nf && i < 6; ++i) a.f[i] = f[i];
        a.nf = std::min(nf, 6);
        a.n = n;
        k_nonfinite<T><<<nsm_ * 4, 256, 0, stream_>>>(a, flag_);
        check(cudaGetLastError(), "k_nonfinite launch");
        int h = 0;
        check(cudaMemcpyAsync(&h, flag_, sizeof(int), cudaMemcpyDeviceToHost, stream_), "cudaMemcpy D2H");
        check(cudaStreamSynchronize(stream_), "sync");
        return h != 0;
    }
    bool any_nonfinite(const double *const *f, int nf, int64_t n) override { return any_nonfinite_t(f, nf, n); }
    bool any_nonfinite(const float *const *f, int nf, int64_t n) override { return any_nonfinite_t(f, nf, n); }

    template <typename T>
    void sources_t(const SourceParams<T> &p)
    {
        if (!p.npts) return;
        use();
        k_sources<T><<<(p.npts + 127) / 128, 128, 0, stream_>>>(p);
        check(cudaGetLastError(), "k_sources launch");
    }
    void sources(const SourceParams<double> &p) override { sources_t(p); }
    void sources(const SourceParams<float> &p) override { sources_t(p); }

    template <typename T>
    void ghosts_t(const GhostParams<T> &p)
    {
        int mu = 1, mv = 1;
        for (int f = 0; f < p.nfaces; ++f)
        {
            mu = max(mu, p.faces[f].u1);
            mv = max(mv, p.faces[f].v1);
        }
        use();
        dim3 block(32, 8);
        dim3 grid((mu + 31) / 32, (mv + 7) / 8, p.nfaces);
        k_ghosts<T><<<grid, block, 0, stream_>>>(p);
        check(cudaGetLastError(), "k_ghosts launch");
    }
    void ghosts(const GhostParams<double> &p) override { ghosts_t(p); }
    void ghosts(const GhostParams<float> &p) override { ghosts_t(p); }

    void probe(const double *f, const int64_t *lin, const double *w, int n, double *out) override
    {
        use();
        k_probe<double><<<1, 1, 0, stream_>>>(f, lin, w, n, out);
        check(cudaGetLastError(), "k_probe launch");
    }
    void probe(const float *f, const int64_t *lin, const double *w, int n, double *out) override
    {
        use();
        k_probe<float><<<1, 1, 0, stream_>>>(f, lin, w, n, out);
        check(cudaGetLastError(), "k_probe launch");
    }
    void dft_norm(const double *re, const double *im, int64_t n, double *out) override
    {
        use();
        k_dft_norm<<<1, 256, 0, stream_>>>(re, im, n, out);
        check(cudaGetLastError(), "k_dft_norm launch");
    }
    const char *name() const override { return "cuda"; }
    double timed(const std::function<void()> &f) override
    {
        use();
        cudaEvent_t a, b;
        check(cudaEventCreate(&a), "cudaEventCreate");
        check(cudaEventCreate(&b), "cudaEventCreate");
        float ms = 0;
        try
        {
            check(cudaEventRecord(a, stream_), "cudaEventRecord");
            f();
                check(cudaEventRecord(b, stream_), "cudaEventRecord");
            check(cudaEventSynchronize(b), "cudaEventSynchronize");
            check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
            check_err();
        }
        catch (...)
        {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            throw;
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return ms;
    }
    void time_passes(bool on) override { time_pass_ = on; }
    double pass_ms() override
    {
        use();
        const double ms = pass_acc_ + drain_passes();
        pass_acc_ = 0;
        return ms;
    }
    // summed elapsed time of the event pairs in use; frees them
    double drain_passes()
    {
        double ms = 0;
        for (size_t i = 0; i < pass_n_; ++i)
        {
            float t = 0;
            check(cudaEventSynchronize(pass_ev_[i].second), "cudaEventSynchronize");
            check(cudaEventElapsedTime(&t, pass_ev_[i].first, pass_ev_[i].second), "cudaEventElapsedTime");
            ms += t;
        }
        pass_n_ = 0;
        return ms;
    }
    // the handle's stream, ordered after the DFT sums already issued
    cudaStream_t stream()
    {
        use();
        return stream_;
    }

private:
    cudaStream_t stream_{nullptr};
    int dev_{0};
    int *err_{nullptr};
    int *flag_{nullptr};  // result word of the divergence check
    std::map<std::tuple<const void *, int, int>, CUtensorMap> maps_;
    std::map<std::string, Jobs> jobs_;
    std::vector<std::string> jobs_order_;  // keys of jobs_, oldest first
    static constexpr size_t kJobCache = 8;
    cudaStream_t side_{nullptr};
    int nsm_{0};
    cudaEvent_t fork_{nullptr}, join_{nullptr}, face_h_{nullptr};
    // timing events of the fused passes (time_passes / pass_ms): pairs in
    // use and the pool, reused across calls
    static constexpr size_t kPassEvents = 1024;
    bool time_pass_{false};
    size_t pass_n_{0};
    double pass_acc_{0};
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pass_ev_;
};
} // namespace

Backend *new_default_backend(int device) { return new CudaBackend(device); }

void *backend_stream(Backend *be)
{
    auto *cb = dynamic_cast<CudaBackend *>(be);
    return cb ? (void *)cb->stream() : nullptr;
}
} // namespace ffipg
