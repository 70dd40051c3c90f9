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
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
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

// ---------------------------------------------------------------------------
// k_sg_gemm_tc: the same product on the 5th-generation tensor cores, for
// operands whose reduction index K is contiguous (A[m][k] row-major, B read
// as B^T[n][k]): 128 x 128 output tiles, K in steps of 64.  One thread (warp
// 0) streams the A and B tiles into a 4-stage ring by TMA
// (cp.async.bulk.tensor.2d, 128-byte swizzle: each tile row is one 128-byte
// swizzle row, 8 rows one 1024-byte atom); one thread (warp 1) issues
// tcgen05.mma (kind::f16, bf16 x bf16 -> fp32, M = 128, N = 128, K = 16 per
// instruction) into a 128-lane x 128-column fp32 accumulator in tensor
// memory, and tcgen05.commit returns each stage to the producer once the
// MMAs reading it are done; then the four warps read their 32 accumulator
// lanes (tcgen05.ld) and write C (+ bias, or C +=).  Every mbarrier wait is
// bounded (global timer); a wait that gives up sets *err and the CTA drains
// its copies and MMAs (bounded) before it frees the tensor memory.
constexpr int TC_M = 128, TC_N = 128, TC_K = 64, TC_STAGES = 4;
constexpr int TC_A_BYTES = TC_M * TC_K * 2, TC_B_BYTES = TC_N * TC_K * 2;
constexpr int TC_SMEM = 1024 + TC_STAGES * (TC_A_BYTES + TC_B_BYTES) + 256;
constexpr uint64_t kTcWaitNs = 2000000000ull;

struct TcArgs
{
    CUtensorMap ta;  // A: dims (K, M), box (64, 128), 128-byte swizzle
    CUtensorMap tb;  // B^T: dims (K, N), box (64, 128), 128-byte swizzle
    int M, N, K;
    float *C;
    int64_t crs, ccs;
    const float *bias;
    int accumulate;
    int *err;
};

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool tc_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t tc_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// waits for the phase `parity` of the mbarrier; false once limit_ns passed
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns)
{
    if (tc_try_wait(bar, parity)) return true;
    const uint64_t t0 = tc_ns();
    for (;;)
    {
        if (tc_try_wait(bar, parity)) return true;
        if (tc_ns() - t0 > limit_ns) return false;
    }
}

// shared-memory matrix descriptor of a K-major tile in the 128-byte swizzle
// layout: start address, leading byte offset 16 (unused by this layout),
// stride byte offset 1024 (8 rows of 128 bytes), descriptor version 1,
// layout type 2 (128-byte swizzle)
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
           ((uint64_t)2 << 61);
}

// instruction descriptor of kind::f16: D fp32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

__global__ void __launch_bounds__(128, 1) k_sg_gemm_tc(const __grid_constant__ TcArgs P)
{
    extern __shared__ uint8_t tc_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sa = smem, *sb = smem + TC_STAGES * TC_A_BYTES;
    uint64_t *full = (uint64_t *)(sb + TC_STAGES * TC_B_BYTES), *empty = full + TC_STAGES, *done = empty + TC_STAGES;
    uint32_t *tslot = (uint32_t *)(done + 1);
    int *cta_err = (int *)(tslot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * TC_M, n0 = blockIdx.x * TC_N;
    const int nk = (P.K + TC_K - 1) / TC_K;
    if (threadIdx.x == 0)
    {
        for (int s = 0; s < TC_STAGES; ++s)
        {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&full[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&empty[s])) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(done)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *cta_err = 0;
    }
    if (warp == 0)
    {
        // TMEM: 128 columns of 128 lanes x 32 bit, the fp32 accumulator
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tslot)), "r"(TC_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    if (threadIdx.x == 0)
    {
        // producer: stage s of tile kb, after the MMAs of tile kb - STAGES freed it
        int issued = 0;
        for (int kb = 0; kb < nk; ++kb)
        {
            const int s = kb % TC_STAGES;
            if (kb >= TC_STAGES && !tc_wait(tc_smem(&empty[s]), ((kb / TC_STAGES) - 1) & 1, kTcWaitNs))
            {
                atomicExch(cta_err, 1);
                break;
            }
            if (*(volatile int *)cta_err) break;
            const uint32_t fb = tc_smem(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(TC_A_BYTES + TC_B_BYTES)
                         : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                    tc_smem(sa + s * TC_A_BYTES)),
                "l"((uint64_t)&P.ta), "r"(kb * TC_K), "r"(m0), "r"(fb)
                : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                    tc_smem(sb + s * TC_B_BYTES)),
                "l"((uint64_t)&P.tb), "r"(kb * TC_K), "r"(n0), "r"(fb)
                : "memory");
            issued = kb + 1;
        }
        // drain: every issued copy has landed before the CTA may leave
        for (int kb = (issued > TC_STAGES ? issued - TC_STAGES : 0); kb < issued; ++kb)
            if (!tc_wait(tc_smem(&full[kb % TC_STAGES]), (kb / TC_STAGES) & 1, kTcWaitNs)) atomicExch(cta_err, 1);
    }
    else if (threadIdx.x == 32)
    {
        // MMA issuer
        for (int kb = 0; kb < nk; ++kb)
        {
            const int s = kb % TC_STAGES;
            if (!tc_wait(tc_smem(&full[s]), (kb / TC_STAGES) & 1, kTcWaitNs))
            {
                atomicExch(cta_err, 1);
                break;
            }
            if (*(volatile int *)cta_err) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = tc_smem(sa + s * TC_A_BYTES), b0 = tc_smem(sb + s * TC_B_BYTES);
#pragma unroll
            for (int k = 0; k < TC_K / 16; ++k)
            {
                const uint64_t da = tc_desc(a0 + 32 * k), db = tc_desc(b0 + 32 * k);
                const uint32_t acc = (kb > 0 || k > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(kTcIdesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(&empty[s]))
                         : "memory");
        }
        // the accumulator is complete once every MMA issued above is
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(done))
                     : "memory");
    }
    __syncwarp();
    const bool ok = tc_wait(tc_smem(done), 0, kTcWaitNs);
    if (!ok) atomicExch(cta_err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    const bool good = ok && !*(volatile int *)cta_err && nk > 0;
    // epilogue: warp w reads accumulator lanes 32 w .. 32 w + 31 (tile rows)
    const int m = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < TC_N && good; c0 += 8)
    {
        uint32_t r[8];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                     : "r"(taddr)
                     : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (m < P.M)
        {
            const float b = P.bias ? P.bias[m] : 0.f;
#pragma unroll
            for (int j = 0; j < 8; ++j)
            {
                const int n = n0 + c0 + j;
                if (n >= P.N) continue;
                float v = __uint_as_float(r[j]);
                if (P.bias) v += b;
                float &dst = P.C[m * P.crs + n * P.ccs];
                dst = P.accumulate ? dst + v : v;
            }
        }
    }
    if (!good && threadIdx.x == 0) atomicExch(P.err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N) : "memory");
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

// the transposed column matrix colsT[N*Do*Ho*Wo][C*kd*kh*kw] (the reduction
// index of the forward GEMM contiguous, as the tcgen05 kernel reads it)
__global__ void k_sg_im2col_t(ConvGeom G, const __nv_bfloat16 *x, __nv_bfloat16 *colsT)
{
    const int64_t P = (int64_t)G.Do * G.Ho * G.Wo, NP = P * G.N;
    const int64_t rows = (int64_t)G.C * G.kd * G.kh * G.kw;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= rows * NP) return;
    const int64_t col = t / rows, row = t % rows;
    const int kw = (int)(row % G.kw), kh = (int)((row / G.kw) % G.kh), kd = (int)((row / (G.kw * G.kh)) % G.kd);
    const int c = (int)(row / ((int64_t)G.kw * G.kh * G.kd));
    const int n = (int)(col / P);
    const int64_t p = col % P;
    const int ow = (int)(p % G.Wo), oh = (int)((p / G.Wo) % G.Ho), od = (int)(p / ((int64_t)G.Wo * G.Ho));
    const int id = od * G.sd - G.pd + kd, ih = oh * G.sh - G.ph + kh, iw = ow * G.sw - G.pw + kw;
    __nv_bfloat16 v = __float2bfloat16(0.f);
    if (id >= 0 && id < G.D && ih >= 0 && ih < G.H && iw >= 0 && iw < G.W)
        v = x[((((int64_t)n * G.C + c) * G.D + id) * G.H + ih) * G.W + iw];
    colsT[t] = v;
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

namespace
{
// cuTensorMapEncodeTiled from the driver, without linking libcuda
PFN_cuTensorMapEncodeTiled_v12000 tc_encode()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        check(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q),
              "cudaGetDriverEntryPoint(cuTensorMapEncodeTiled)");
        if (q != cudaDriverEntryPointSuccess || !p) throw std::runtime_error("cuTensorMapEncodeTiled not available");
        fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// a K-contiguous bf16 operand: rows of K elements, `rows` of them, row stride
// rs elements; box 64 x 128 in the 128-byte swizzle
CUtensorMap tc_map(const void *base, int K, int rows, int64_t rs)
{
    CUtensorMap m;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)rs * 2};
    cuuint32_t box[2] = {(cuuint32_t)TC_K, 128u};
    cuuint32_t es[2] = {1, 1};
    CUresult r = tc_encode()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

// per device: the error word of the tensor-core GEMM (a bounded wait gave
// up) and whether its shared-memory attribute is set
struct TcDevice
{
    int *err{nullptr};
    bool attr{false};
};
std::mutex tc_mu;
TcDevice tc_dev[64];

TcDevice &tc_device()
{
    int d = 0;
    check(cudaGetDevice(&d), "cudaGetDevice");
    if (d < 0 || d >= 64) throw std::runtime_error("device index beyond 63");
    std::lock_guard<std::mutex> g(tc_mu);
    TcDevice &T = tc_dev[d];
    if (!T.err)
    {
        check(cudaMalloc(&T.err, sizeof(int)), "cudaMalloc");
        check(cudaMemset(T.err, 0, sizeof(int)), "cudaMemset");
    }
    if (!T.attr)
    {
        check(cudaFuncSetAttribute(k_sg_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM), "cudaFuncSetAttribute");
        T.attr = true;
    }
    return T;
}
} // namespace

bool sg_gemm_tc_eligible(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs)
{
    return M > 0 && N > 0 && K > 0 && acs == 1 && brs == 1 && ars > 0 && bcs > 0 && ars % 8 == 0 && bcs % 8 == 0 &&
           ((uintptr_t)A & 15) == 0 && ((uintptr_t)B & 15) == 0 && ars < (int64_t(1) << 36) && bcs < (int64_t(1) << 36) &&
           (M + TC_M - 1) / TC_M <= 65535;
}

int sg_gemm_tc(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs, float *C,
               int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream)
{
    if (!sg_gemm_tc_eligible(M, N, K, A, ars, acs, B, brs, bcs))
        throw std::invalid_argument("tensor-core GEMM: needs M, N, K >= 1, A[m][k] and B[k][n] with k contiguous, row strides "
                                    "multiples of 8 elements and 16-byte aligned operands");
    TcDevice &T = tc_device();
    TcArgs P;
    P.ta = tc_map(A, K, M, ars);
    P.tb = tc_map(B, K, N, bcs);
    P.M = M;
    P.N = N;
    P.K = K;
    P.C = C;
    P.crs = crs;
    P.ccs = ccs;
    P.bias = bias;
    P.accumulate = accumulate;
    P.err = T.err;
    dim3 grid((N + TC_N - 1) / TC_N, (M + TC_M - 1) / TC_M);
    k_sg_gemm_tc<<<grid, 128, TC_SMEM, (cudaStream_t)stream>>>(P);
    check(cudaGetLastError(), "k_sg_gemm_tc launch");
    return 0;
}

int sg_check()
{
    int d = 0;
    check(cudaGetDevice(&d), "cudaGetDevice");
    int *err = nullptr;
    {
        std::lock_guard<std::mutex> g(tc_mu);
        if (d >= 0 && d < 64) err = tc_dev[d].err;
    }
    check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    if (!err) return 0;
    int h = 0;
    check(cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (h)
    {
        check(cudaMemset(err, 0, sizeof(int)), "cudaMemset");
        throw std::runtime_error("tensor-core GEMM: a wait on its TMA ring or its MMAs timed out");
    }
    return 0;
}

int sg_gemm(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs, float *C,
            int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream, int path)
{
    if (M < 0 || N < 0 || K < 0) throw std::invalid_argument("negative GEMM size");
    if (path < 0 || path > 2) throw std::invalid_argument("GEMM path must be 0 (auto), 1 (tcgen05) or 2 (mma.sync)");
    if (!M || !N) return 0;
    // K-contiguous operands go to the tensor-core (tcgen05) kernel
    if (path == 1 || (path == 0 && sg_gemm_tc_eligible(M, N, K, A, ars, acs, B, brs, bcs)))
        return sg_gemm_tc(M, N, K, A, ars, acs, B, brs, bcs, C, crs, ccs, bias, accumulate, stream);
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

int sg_im2col_t(const void *x, const int *shape, const int *kernel, const int *stride, const int *pad, void *colsT, void *stream)
{
    const ConvGeom G = make_geom(shape, kernel, stride, pad);
    const int64_t total = (int64_t)G.C * G.kd * G.kh * G.kw * G.N * G.Do * G.Ho * G.Wo;
    k_sg_im2col_t<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(G, (const __nv_bfloat16 *)x,
                                                                                     (__nv_bfloat16 *)colsT);
    check(cudaGetLastError(), "k_sg_im2col_t launch");
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
