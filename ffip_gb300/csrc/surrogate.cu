// Kernels of the design-screening surrogate (a small 3-D/2-D convolutional
// network trained on this project's own FDTD runs; see
// ffip_gb300/surrogate.py).  Convolutions run as im2col + GEMM:
//
//   k_sg_gemm     C[M,N] (fp32) = A[M,K] B[K,N] (+ bias[M]) (or C +=), A and B
//                 bf16 with arbitrary row / column strides, on the tensor
//                 cores with mma.sync m16n8k16 (bf16 in, fp32 accumulate);
//                 64 x 64 x 32 block tiles, 4 warps of 32 x 32
//   k_sg_im2col   x[N,C,D,H,W] -> cols[C*kd*kh*kw, N*Do*Ho*Wo] (bf16)
//   k_sg_col2im   the transpose (gather form, fp32 in, fp32 out, no atomics)
//
// The network is small (about 5 M parameters): these kernels aim at being
// exact and simple, not at the tensor cores' peak.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>

namespace ffipg
{
namespace
{
void check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

constexpr int BM = 64, BN = 64, BK = 32, PADK = 8;

__device__ __forceinline__ uint32_t pack2(const __nv_bfloat16 *p)
{
    return *reinterpret_cast<const uint32_t *>(p);
}

__global__ void __launch_bounds__(128) k_sg_gemm(int M, int N, int K, const __nv_bfloat16 *A, int64_t ars, int64_t acs,
                                                 const __nv_bfloat16 *B, int64_t brs, int64_t bcs, float *C, int64_t crs,
                                                 int64_t ccs, const float *bias, int accumulate)
{
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PADK];  // [m][k]
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PADK];  // [n][k]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, tig = lane & 3;
    const int wm = warp >> 1, wn = warp & 1;  // 2 x 2 warps of 32 x 32
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int t = 0; t < 4; ++t) acc[i][j][t] = 0.f;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int k0 = 0; k0 < K; k0 += BK)
    {
        // stage the A and B tiles (bounds-checked, zero filled); consecutive
        // threads walk the operand's unit-stride direction so that the
        // global loads coalesce
        if (acs == 1)
            for (int e = tid; e < BM * BK; e += 128)
            {
                const int r = e / BK, c = e % BK, m = m0 + r, k = k0 + c;
                As[r][c] = (m < M && k < K) ? A[m * ars + k] : zero;
            }
        else
            for (int e = tid; e < BM * BK; e += 128)
            {
                const int r = e % BM, c = e / BM, m = m0 + r, k = k0 + c;
                As[r][c] = (m < M && k < K) ? A[m * ars + k * acs] : zero;
            }
        if (bcs == 1)
            for (int e = tid; e < BN * BK; e += 128)
            {
                const int r = e % BN, c = e / BN, n = n0 + r, k = k0 + c;
                Bs[r][c] = (n < N && k < K) ? B[k * brs + n] : zero;
            }
        else
            for (int e = tid; e < BN * BK; e += 128)
            {
                const int r = e / BK, c = e % BK, n = n0 + r, k = k0 + c;
                Bs[r][c] = (n < N && k < K) ? B[k * brs + n * bcs] : zero;
            }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16)
        {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
            {
                const int r = wm * 32 + i * 16 + g;
                a[i][0] = pack2(&As[r][kk + 2 * tig]);
                a[i][1] = pack2(&As[r + 8][kk + 2 * tig]);
                a[i][2] = pack2(&As[r][kk + 2 * tig + 8]);
                a[i][3] = pack2(&As[r + 8][kk + 2 * tig + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
            {
                const int n = wn * 32 + j * 8 + g;
                b[j][0] = pack2(&Bs[n][kk + 2 * tig]);
                b[j][1] = pack2(&Bs[n][kk + 2 * tig + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                        "{%0,%1,%2,%3};"
                        : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
                        : "r"(a[i][0]), "r"(a[i][1]), "r"(a[i][2]), "r"(a[i][3]), "r"(b[j][0]), "r"(b[j][1]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int t = 0; t < 4; ++t)
            {
                const int m = m0 + wm * 32 + i * 16 + g + (t >= 2 ? 8 : 0);
                const int n = n0 + wn * 32 + j * 8 + 2 * tig + (t & 1);
                if (m >= M || n >= N) continue;
                float v = acc[i][j][t];
                if (bias) v += bias[m];
                float &dst = C[m * crs + n * ccs];
                dst = accumulate ? dst + v : v;
            }
}

struct ConvGeom
{
    int N, C, D, H, W;     // input
    int kd, kh, kw;        // kernel
    int sd, sh, sw;        // stride
    int pd, ph, pw;        // padding
    int Do, Ho, Wo;        // output
};

__global__ void k_sg_im2col(ConvGeom G, const __nv_bfloat16 *x, __nv_bfloat16 *cols)
{
    const int64_t P = (int64_t)G.Do * G.Ho * G.Wo, NP = P * G.N;
    const int64_t rows = (int64_t)G.C * G.kd * G.kh * G.kw;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= rows * NP) return;
    const int64_t row = t / NP, col = t % NP;
    const int kw = (int)(row % G.kw), kh = (int)((row / G.kw) % G.kh), kd = (int)((row / (G.kw * G.kh)) % G.kd);
    const int c = (int)(row / ((int64_t)G.kw * G.kh * G.kd));
    const int n = (int)(col / P);
    const int64_t p = col % P;
    const int ow = (int)(p % G.Wo), oh = (int)((p / G.Wo) % G.Ho), od = (int)(p / ((int64_t)G.Wo * G.Ho));
    const int id = od * G.sd - G.pd + kd, ih = oh * G.sh - G.ph + kh, iw = ow * G.sw - G.pw + kw;
    __nv_bfloat16 v = __float2bfloat16(0.f);
    if (id >= 0 && id < G.D && ih >= 0 && ih < G.H && iw >= 0 && iw < G.W)
        v = x[((((int64_t)n * G.C + c) * G.D + id) * G.H + ih) * G.W + iw];
    cols[t] = v;
}

__global__ void k_sg_col2im(ConvGeom G, const float *dcols, float *dx)
{
    const int64_t P = (int64_t)G.Do * G.Ho * G.Wo, NP = P * G.N;
    const int64_t total = (int64_t)G.N * G.C * G.D * G.H * G.W;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int iw = (int)(t % G.W), ih = (int)((t / G.W) % G.H), id = (int)((t / ((int64_t)G.W * G.H)) % G.D);
    const int c = (int)((t / ((int64_t)G.W * G.H * G.D)) % G.C), n = (int)(t / ((int64_t)G.W * G.H * G.D * G.C));
    float s = 0.f;
    for (int kd = 0; kd < G.kd; ++kd)
    {
        const int a = id + G.pd - kd;
        if (a < 0 || a % G.sd) continue;
        const int od = a / G.sd;
        if (od >= G.Do) continue;
        for (int kh = 0; kh < G.kh; ++kh)
        {
            const int b = ih + G.ph - kh;
            if (b < 0 || b % G.sh) continue;
            const int oh = b / G.sh;
            if (oh >= G.Ho) continue;
            for (int kw = 0; kw < G.kw; ++kw)
            {
                const int e = iw + G.pw - kw;
                if (e < 0 || e % G.sw) continue;
                const int ow = e / G.sw;
                if (ow >= G.Wo) continue;
                const int64_t row = (((int64_t)c * G.kd + kd) * G.kh + kh) * G.kw + kw;
                const int64_t col = (int64_t)n * P + ((int64_t)od * G.Ho + oh) * G.Wo + ow;
                s += dcols[row * NP + col];
            }
        }
    }
    dx[t] = s;
}

ConvGeom make_geom(const int *shape, const int *kernel, const int *stride, const int *pad)
{
    ConvGeom G;
    G.N = shape[0]; G.C = shape[1]; G.D = shape[2]; G.H = shape[3]; G.W = shape[4];
    G.kd = kernel[0]; G.kh = kernel[1]; G.kw = kernel[2];
    G.sd = stride[0]; G.sh = stride[1]; G.sw = stride[2];
    G.pd = pad[0]; G.ph = pad[1]; G.pw = pad[2];
    if (G.N < 1 || G.C < 1 || G.D < 1 || G.H < 1 || G.W < 1 || G.kd < 1 || G.kh < 1 || G.kw < 1 || G.sd < 1 || G.sh < 1 ||
        G.sw < 1 || G.pd < 0 || G.ph < 0 || G.pw < 0)
        throw std::invalid_argument("bad convolution geometry");
    G.Do = (G.D + 2 * G.pd - G.kd) / G.sd + 1;
    G.Ho = (G.H + 2 * G.ph - G.kh) / G.sh + 1;
    G.Wo = (G.W + 2 * G.pw - G.kw) / G.sw + 1;
    if (G.Do < 1 || G.Ho < 1 || G.Wo < 1) throw std::invalid_argument("convolution output is empty");
    return G;
}
} // namespace

int sg_gemm(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs, float *C,
            int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream)
{
    if (M < 0 || N < 0 || K < 0) throw std::invalid_argument("negative GEMM size");
    if (!M || !N) return 0;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    if (grid.y > 65535) throw std::invalid_argument("GEMM M too large");
    k_sg_gemm<<<grid, 128, 0, (cudaStream_t)stream>>>(M, N, K, (const __nv_bfloat16 *)A, ars, acs, (const __nv_bfloat16 *)B, brs,
                                                    bcs, C, crs, ccs, bias, accumulate);
    check(cudaGetLastError(), "k_sg_gemm launch");
    return 0;
}

int sg_im2col(const void *x, const int *shape, const int *kernel, const int *stride, const int *pad, void *cols, void *stream)
{
    const ConvGeom G = make_geom(shape, kernel, stride, pad);
    const int64_t total = (int64_t)G.C * G.kd * G.kh * G.kw * G.N * G.Do * G.Ho * G.Wo;
    k_sg_im2col<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(G, (const __nv_bfloat16 *)x,
                                                                                   (__nv_bfloat16 *)cols);
    check(cudaGetLastError(), "k_sg_im2col launch");
    return 0;
}

int sg_col2im(const float *dcols, const int *shape, const int *kernel, const int *stride, const int *pad, float *dx, void *stream)
{
    const ConvGeom G = make_geom(shape, kernel, stride, pad);
    const int64_t total = (int64_t)G.N * G.C * G.D * G.H * G.W;
    k_sg_col2im<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(G, dcols, dx);
    check(cudaGetLastError(), "k_sg_col2im launch");
    return 0;
}
} // namespace ffipg
