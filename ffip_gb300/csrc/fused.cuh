// Fused H+E time step: one z-marching pass over the grid per time step.
//
// Each CTA owns a TX x TY tile in (x, y) and marches a chunk of z planes.
// For plane k it needs E(k), E(k+1) and H(k) of the previous time level;
// those planes are staged into shared memory by TMA (cp.async.bulk.tensor,
// one 3-D tensor map per field array) through an S-stage ring completed by
// mbarriers, so the loads of later planes are in flight while plane k is
// computed.  Per plane:
//   1. H(k) at the new level is computed on the tile plus a one-point halo on
//      the low x and y sides (the halo points belong to neighbouring CTAs and
//      are recomputed here, not written) and kept in shared memory;
//   2. E(k) at the new level is computed on the tile from H(k) and H(k-1)
//      (the previous plane's result, still in shared memory).
// Every field value is read from HBM once and written once per time step.
// Because neighbouring CTAs read the previous level while this CTA writes the
// new one, field buffers (and the H-side CPML psi) ping-pong between steps;
// E-side CPML psi and polarisation state are only touched by their owner and
// are updated in place.  Each chunk starts by recomputing H of the plane
// below it (no writes).  Only used with "None" boundaries on every face and no
// magnetic poles (the engine checks this).
//
// The per-point arithmetic is the same code the separate H/E kernels use
// (stencil.cuh: curl_term, material_point, dft_point), so both passes give
// identical results.  Every mbarrier wait is bounded; on timeout the kernel
// records an error code, waits (bounded) for its outstanding copies and
// returns.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.hpp"

namespace ffipg
{
template <typename T>
struct FusedShape;
template <>
struct FusedShape<float>
{
    static constexpr int TX = 32, TY = 8, XOFF = 4, BX = 40, S = 4;
};
template <>
struct FusedShape<double>
{
    static constexpr int TX = 32, TY = 8, XOFF = 2, BX = 36, S = 3;
};

template <typename T>
struct FusedLayout
{
    using SH = FusedShape<T>;
    static constexpr int E_BYTES = (SH::TY + 2) * SH::BX * (int)sizeof(T);  // one E box
    static constexpr int H_BYTES = (SH::TY + 1) * SH::BX * (int)sizeof(T);  // one H box
    static constexpr int E_TILE = (E_BYTES + 127) / 128 * 128;
    static constexpr int H_TILE = (H_BYTES + 127) / 128 * 128;
    static constexpr int STAGE = 3 * E_TILE + 3 * H_TILE;
    static constexpr int TX_BYTES = 3 * E_BYTES + 3 * H_BYTES;  // bytes one stage receives
    static constexpr int HN_OFF = 128 + SH::S * STAGE;
    static constexpr int HN_PLANE = 3 * (SH::TY + 1) * (SH::TX + 1);  // elements of one H ring plane
    static constexpr int SMEM = HN_OFF + 2 * HN_PLANE * (int)sizeof(T);
};

template <typename T>
struct FusedLaunch
{
    CUtensorMap tm_e[3];  // E input arrays, box (BX, TY + 2, 1)
    CUtensorMap tm_h[3];  // H input arrays, box (BX, TY + 1, 1)
    FusedParams<T> fp;
    int kchunk;
    int *err;             // set to a non-zero code when a wait times out
};

constexpr int kFusedWaitLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    for (int i = 0; i < kFusedWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

template <typename T>
__global__ void __launch_bounds__(256) k_fused(const __grid_constant__ FusedLaunch<T> L)
{
    using SH = FusedShape<T>;
    using LY = FusedLayout<T>;
    constexpr int TX = SH::TX, TY = SH::TY, XOFF = SH::XOFF, BX = SH::BX, S = SH::S;
    extern __shared__ __align__(128) unsigned char smem[];
    const FusedParams<T> &F = L.fp;
    const SideParams<T> &PH = F.h;
    const SideParams<T> &PE = F.e;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * L.kchunk;
    const int k1 = min(k0 + L.kchunk, PE.Mz);
    const int NP = k1 - k0 + 2;  // planes k0-1 .. k1
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    T *hn = reinterpret_cast<T *>(smem + LY::HN_OFF);
    auto e_tile = [&](int st, int c) { return reinterpret_cast<const T *>(smem + 128 + st * LY::STAGE + c * LY::E_TILE); };
    auto h_tile = [&](int st, int c) {
        return reinterpret_cast<const T *>(smem + 128 + st * LY::STAGE + 3 * LY::E_TILE + c * LY::H_TILE);
    };
    auto hn_at = [&](int ring, int c, int row, int col) -> T & { return hn[ring * LY::HN_PLANE + (c * (TY + 1) + row) * (TX + 1) + col]; };

    if (tid == 0)
    {
        for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    auto issue = [&](int p) {
        const int st = p % S, z = k0 - 1 + p;
        mbar_expect_tx(&bar[st], LY::TX_BYTES);
        unsigned char *base = smem + 128 + st * LY::STAGE;
        for (int c = 0; c < 3; ++c) tma_load_3d(base + c * LY::E_TILE, &L.tm_e[c], x0 - XOFF, y0 - 1, z, &bar[st]);
        for (int c = 0; c < 3; ++c) tma_load_3d(base + 3 * LY::E_TILE + c * LY::H_TILE, &L.tm_h[c], x0 - XOFF, y0 - 1, z, &bar[st]);
    };
    int issued = min(S, NP);
    if (tid == 0)
        for (int p = 0; p < issued; ++p) issue(p);

    const int64_t sy = PE.sy, sz = PE.sz;

    // H at the new level for point (x, y) of plane k, own H component c;
    // stE0 / stE1: stages holding planes k / k+1.  Reads E and H of the old
    // level from shared memory.
    auto h_value = [&](int c, int x, int y, int k, int stE0, int stE1, bool owned, T &out_v) -> bool {
        if (x < PH.vlo[c][0] || x > PH.vhi[c][0] || y < PH.vlo[c][1] || y > PH.vhi[c][1] || k < PH.vlo[c][2] || k > PH.vhi[c][2])
            return false;
        const int r = y - (y0 - 1), col = x - (x0 - XOFF);
        const T *E0x = e_tile(stE0, 0), *E0y = e_tile(stE0, 1), *E0z = e_tile(stE0, 2);
        T curl1, curl2;
        if (c == 0)  // Hx: -(dEz/dy) + dEy/dz
        {
            curl1 = (E0z[r * BX + col] - E0z[(r + 1) * BX + col]) * PH.inv_dx;
            curl2 = (E0y[r * BX + col] - e_tile(stE1, 1)[r * BX + col]) * PH.inv_dx;
        }
        else if (c == 1)  // Hy: -(dEx/dz) + dEz/dx
        {
            curl1 = (E0x[r * BX + col] - e_tile(stE1, 0)[r * BX + col]) * PH.inv_dx;
            curl2 = (E0z[r * BX + col] - E0z[r * BX + col + 1]) * PH.inv_dx;
        }
        else  // Hz: -(dEy/dx) + dEx/dy
        {
            curl1 = (E0y[r * BX + col] - E0y[r * BX + col + 1]) * PH.inv_dx;
            curl2 = (E0x[r * BX + col] - E0x[(r + 1) * BX + col]) * PH.inv_dx;
        }
        const int64_t idx = (int64_t)x + y * sy + (int64_t)k * sz;
        const int ii[3] = {x, y, k};
        const T term = curl_term(PH, c, ii, idx, curl1, curl2, const_cast<T *>(F.psih_in[c][0]), const_cast<T *>(F.psih_in[c][1]),
                                 owned ? F.psih_out[c][0] : nullptr, owned ? F.psih_out[c][1] : nullptr);
        const T old = h_tile(stE0, c)[r * BX + col];
        T vd;
        material_point(PH, c, x, y, k, idx, old, term, &out_v, &vd);
        if (owned)
        {
            F.hout[c][idx] = out_v;
            if (PH.nunits) dft_point<T>(PH.nunits, PH.units, PH.phase, 3 + c, x, y, k, (double)out_v, (double)vd);
        }
        return true;
    };

    for (int q = 0; q + 1 < NP; ++q)
    {
        const int stA = q % S, stB = (q + 1) % S;
        bool ok = mbar_wait_bounded(&bar[stA], (q / S) & 1) && mbar_wait_bounded(&bar[stB], ((q + 1) / S) & 1);
        if (__syncthreads_or(!ok))
        {
            if (tid == 0)
            {
                atomicExch(L.err, 1);
                for (int p = q; p < issued; ++p) mbar_wait_bounded(&bar[p % S], (p / S) & 1);
            }
            return;
        }
        const int k = k0 - 1 + q;
        const bool owned = q >= 1;
        const int ring = q & 1;
        // 1. H(k) on the tile
        {
            const int x = x0 + tx, y = y0 + ty;
            for (int c = 0; c < 3; ++c)
            {
                T v = T(0);
                if (!h_value(c, x, y, k, stA, stB, owned, v)) v = T(0);
                hn_at(ring, c, ty + 1, tx + 1) = v;
            }
        }
        // ... and on the low-x column and low-y row (recomputed, not written)
        if (tid < TX + TY)
        {
            const int x = tid < TX ? x0 + tid : x0 - 1;
            const int y = tid < TX ? y0 - 1 : y0 + (tid - TX);
            const int row = y - (y0 - 1), col = x - (x0 - 1);
            for (int c = 0; c < 3; ++c)
            {
                T v = T(0);
                if (x < 0 || y < 0 || !h_value(c, x, y, k, stA, stB, false, v)) v = T(0);
                hn_at(ring, c, row, col) = v;
            }
        }
        __syncthreads();
        // 2. E(k) on the tile from H(k) and H(k-1)
        if (owned)
        {
            const int x = x0 + tx, y = y0 + ty;
            const int row = ty + 1, col = tx + 1, prev = ring ^ 1;
            const int r = y - (y0 - 1), ecol = x - (x0 - XOFF);
            for (int c = 0; c < 3; ++c)
            {
                if (x < PE.vlo[c][0] || x > PE.vhi[c][0] || y < PE.vlo[c][1] || y > PE.vhi[c][1] || k < PE.vlo[c][2] || k > PE.vhi[c][2])
                    continue;
                T curl1, curl2;
                if (c == 0)  // Ex: dHz/dy - dHy/dz
                {
                    curl1 = (hn_at(ring, 2, row, col) - hn_at(ring, 2, row - 1, col)) * PE.inv_dx;
                    curl2 = (hn_at(ring, 1, row, col) - hn_at(prev, 1, row, col)) * PE.inv_dx;
                }
                else if (c == 1)  // Ey: dHx/dz - dHz/dx
                {
                    curl1 = (hn_at(ring, 0, row, col) - hn_at(prev, 0, row, col)) * PE.inv_dx;
                    curl2 = (hn_at(ring, 2, row, col) - hn_at(ring, 2, row, col - 1)) * PE.inv_dx;
                }
                else  // Ez: dHy/dx - dHx/dy
                {
                    curl1 = (hn_at(ring, 1, row, col) - hn_at(ring, 1, row, col - 1)) * PE.inv_dx;
                    curl2 = (hn_at(ring, 0, row, col) - hn_at(ring, 0, row - 1, col)) * PE.inv_dx;
                }
                const int64_t idx = (int64_t)x + y * sy + (int64_t)k * sz;
                const int ii[3] = {x, y, k};
                const T term = curl_term(PE, c, ii, idx, curl1, curl2, PE.psi[c][0], PE.psi[c][1], PE.psi[c][0], PE.psi[c][1]);
                const T old = e_tile(stA, c)[r * BX + ecol];
                T vd;
                const T v = material_point(PE, c, x, y, k, idx, old, term, &F.eout[c][idx], &vd);
                if (PE.nunits) dft_point<T>(PE.nunits, PE.units, PE.phase, c, x, y, k, (double)v, (double)vd);
            }
        }
        __syncthreads();
        if (tid == 0 && q + S < NP)
        {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(q + S);
            issued = q + S + 1;
        }
    }
}

} // namespace ffipg
