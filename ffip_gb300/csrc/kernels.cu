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
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "engine.hpp"
#include "fused.cuh"

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
    for (int k = k0; k < k1; ++k)
    {
#pragma unroll
        for (int c = 0; c < 3; ++c)
        {
            if (i < p.vlo[c][0] || i > p.vhi[c][0] || j < p.vlo[c][1] || j > p.vhi[c][1] || k < p.vlo[c][2] || k > p.vhi[c][2]) continue;
            update_point<T, IS_E>(p, c, i, j, k);
        }
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
    void zero(void *p, size_t bytes) override { use(); check(cudaMemsetAsync(p, 0, bytes, stream_), "cudaMemsetAsync"); }
    void sync() override { use(); check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize"); }

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

    bool has_fused() const override { return false; }
    void fused(const FusedParams<double> &p) override
    {
        use();
        launch_fused(p, stream_);
        check(cudaGetLastError(), "k_fused launch");
    }
    void fused(const FusedParams<float> &p) override
    {
        use();
        launch_fused(p, stream_);
        check(cudaGetLastError(), "k_fused launch");
    }

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
    cudaStream_t stream() const { return stream_; }

private:
    cudaStream_t stream_{nullptr};
    int dev_{0};
};
} // namespace

Backend *new_default_backend(int device) { return new CudaBackend(device); }

void *backend_stream(Backend *be)
{
    auto *cb = dynamic_cast<CudaBackend *>(be);
    return cb ? (void *)cb->stream() : nullptr;
}
} // namespace ffipg
