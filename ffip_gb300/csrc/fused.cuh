// Fused H+E time step: one z-marching pass over the grid per time step.
//
// Each CTA owns a TX x TY tile in (x, y) and marches a chunk of KCH z planes.
// For plane k it needs E(k), E(k+1) and H(k) of the previous time level;
// those planes are staged into shared memory by TMA (cp.async.bulk.tensor,
// one 3-D tensor map per field array) through an S-stage ring completed by
// mbarriers, so the loads of the next planes are in flight while plane k is
// computed.  Per plane:
//   1. H(k) at the new level is computed on the tile, and on the low-x column
//      and low-y row that the tile's E update needs (those halo points belong
//      to neighbouring CTAs and are recomputed here, not written), into a
//      two-plane ring in shared memory;
//   2. E(k) at the new level is computed on the tile from H(k) and H(k-1).
// Every field value is read from HBM once and written once per time step.
// Because neighbouring CTAs read the previous level while this CTA writes the
// new one, field buffers (and the H-side CPML psi) ping-pong between steps;
// E-side CPML psi and polarisation state are only touched by their owner and
// are updated in place.  Each chunk starts by recomputing H of the plane
// below it (no writes).  Used with "None" boundaries on every face and no
// magnetic poles (the engine checks this).
//
// The per-point arithmetic is the same as the separate H/E kernels
// (stencil.cuh: pml_combine, material_at, dft_point), so both passes give the
// same bits.  The CPML tables of the tile's x and y range and of the chunk's
// z range are staged in shared memory; a tile plane with no CPML takes the
// plain curl.  Only thread 0 waits on the mbarriers (bounded); on a timeout
// it records an error word, waits (bounded) for its outstanding copies, and
// the whole CTA returns.
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
    static constexpr int TX = 32, TY = 8, XOFF = 4, BX = 40, S = 4, KCH = 32, MINB = 4;  // CTAs per SM (smem-bound)
};
template <>
struct FusedShape<double>
{
    static constexpr int TX = 32, TY = 8, XOFF = 2, BX = 36, S = 3, KCH = 32, MINB = 3;
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
    static constexpr int NX = SH::TX + 1, NY = SH::TY + 1, NZ = SH::KCH + 2;  // CPML table lengths
    static constexpr int PML_OFF = HN_OFF + 2 * HN_PLANE * (int)sizeof(T);
    static constexpr int PML_ELEMS = 6 * (NX + NY + NZ);  // [parity][b,c,ik][n] per axis
    static constexpr int MASK_OFF = PML_OFF + PML_ELEMS * (int)sizeof(T);
    static constexpr int SMEM = MASK_OFF + NZ * 4;  // per plane: bit r = row y0+r has E slots in the tile
};

template <typename T>
struct FusedLaunch
{
    CUtensorMap tm_e[3];  // E input arrays, box (BX, TY + 2, 1)
    CUtensorMap tm_h[3];  // H input arrays, box (BX, TY + 1, 1)
    FusedParams<T> fp;
    int *err;             // set to 1 when a wait times out
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

// Per-CTA context of the fused pass
template <typename T>
struct FusedCtx
{
    using SH = FusedShape<T>;
    using LY = FusedLayout<T>;
    unsigned char *smem;
    const FusedLaunch<T> *L;
    int x0, y0, k0;
    __device__ __forceinline__ const T *e_tile(int st, int c) const
    {
        return reinterpret_cast<const T *>(smem + 128 + st * LY::STAGE + c * LY::E_TILE);
    }
    __device__ __forceinline__ const T *h_tile(int st, int c) const
    {
        return reinterpret_cast<const T *>(smem + 128 + st * LY::STAGE + 3 * LY::E_TILE + c * LY::H_TILE);
    }
    __device__ __forceinline__ T &hn_at(int ring, int c, int row, int col) const
    {
        return reinterpret_cast<T *>(smem + LY::HN_OFF)[ring * LY::HN_PLANE + (c * (SH::TY + 1) + row) * (SH::TX + 1) + col];
    }
    __device__ __forceinline__ T *pml(int axis) const
    {
        T *base = reinterpret_cast<T *>(smem + LY::PML_OFF);
        return axis == 0 ? base : axis == 1 ? base + 6 * LY::NX : base + 6 * (LY::NX + LY::NY);
    }
    // table entry v (0 = b, 1 = c, 2 = 1/k) of axis A and parity q at
    // position pos (an x, y or k index)
    template <int A>
    __device__ __forceinline__ T pml_val(int q, int v, int pos) const
    {
        constexpr int n = A == 0 ? LY::NX : A == 1 ? LY::NY : LY::NZ;
        const int o = A == 0 ? pos - (x0 - 1) : A == 1 ? pos - (y0 - 1) : pos - (k0 - 1);
        return pml(A)[(q * 3 + v) * n + o];
    }
};

// accdb increment at one point of component GC from its two curls, CPML
// coefficients taken from the staged tables
template <typename T, int GC>
__device__ __forceinline__ T fused_term(const FusedCtx<T> &X, bool pml_plane, int x, int y, int k, int64_t idx, T curl1,
                                        T curl2, const T *pin1, const T *pin2, T *pout1, T *pout2)
{
    using C = CompT<GC>;
    if (!pml_plane) return curl1 - curl2;
    const int p1 = pick<C::a1>(x, y, k), p2 = pick<C::a2>(x, y, k);
    const T cv1 = X.template pml_val<C::a1>(C::q1, 1, p1), cv2 = X.template pml_val<C::a2>(C::q2, 1, p2);
    if (cv1 == T(0) && cv2 == T(0)) return curl1 - curl2;
    return pml_combine(cv1, cv2, X.template pml_val<C::a1>(C::q1, 0, p1), X.template pml_val<C::a2>(C::q2, 0, p2),
                       X.template pml_val<C::a1>(C::q1, 2, p1), X.template pml_val<C::a2>(C::q2, 2, p2), curl1, curl2, pin1,
                       pin2, pout1, pout2, idx);
}

// H at the new level, component GC (3..5), point (x, y) of plane k; stA/stB
// hold planes k/k+1.  Writes the output, psi and DFT only when `owned`.
template <typename T, int GC, bool CHECK>
__device__ __forceinline__ T fused_h(const FusedCtx<T> &X, int x, int y, int k, int stA, int stB, bool owned, bool pml_plane,
                                     bool slots, bool dft)
{
    using SH = FusedShape<T>;
    constexpr int BX = SH::BX, XOFF = SH::XOFF, c = GC - 3;
    const FusedParams<T> &F = X.L->fp;
    const SideParams<T> &PH = F.h;
    if (CHECK && (x < PH.vlo[c][0] || x > PH.vhi[c][0] || y < PH.vlo[c][1] || y > PH.vhi[c][1] || k < PH.vlo[c][2] ||
                  k > PH.vhi[c][2]))
        return T(0);
    const int r = y - (X.y0 - 1), col = x - (X.x0 - XOFF);
    T curl1, curl2;
    if (c == 0)  // Hx: -(dEz/dy) + dEy/dz
    {
        const T *Ez = X.e_tile(stA, 2), *Ey = X.e_tile(stA, 1);
        curl1 = (Ez[r * BX + col] - Ez[(r + 1) * BX + col]) * PH.inv_dx;
        curl2 = (Ey[r * BX + col] - X.e_tile(stB, 1)[r * BX + col]) * PH.inv_dx;
    }
    else if (c == 1)  // Hy: -(dEx/dz) + dEz/dx
    {
        const T *Ex = X.e_tile(stA, 0), *Ez = X.e_tile(stA, 2);
        curl1 = (Ex[r * BX + col] - X.e_tile(stB, 0)[r * BX + col]) * PH.inv_dx;
        curl2 = (Ez[r * BX + col] - Ez[r * BX + col + 1]) * PH.inv_dx;
    }
    else  // Hz: -(dEy/dx) + dEx/dy
    {
        const T *Ey = X.e_tile(stA, 1), *Ex = X.e_tile(stA, 0);
        curl1 = (Ey[r * BX + col] - Ey[r * BX + col + 1]) * PH.inv_dx;
        curl2 = (Ex[r * BX + col] - Ex[(r + 1) * BX + col]) * PH.inv_dx;
    }
    const int idx = x + y * (int)PH.sy + k * (int)PH.sz;
    const T term = fused_term<T, GC>(X, pml_plane, x, y, k, idx, curl1, curl2, F.psih_in[c][0], F.psih_in[c][1],
                                     owned ? F.psih_out[c][0] : nullptr, owned ? F.psih_out[c][1] : nullptr);
    const T old = X.h_tile(stA, c)[r * BX + col];
    T v, vd;
    if (!slots)
    {
        v = old + PH.coef_def * term;
        vd = PH.g_def * v;
    }
    else
        v = material_at(PH, PH.slot[c], slot_of(PH.slot[c], PH.My, x, y, k, idx), old, term, &vd);
    if (owned)
    {
        F.hout[c][idx] = v;
        if (dft) dft_point<T>(PH.nunits, PH.units, PH.phase, GC, x, y, k, (double)v, (double)vd);
    }
    return v;
}

// E at the new level, component GC (0..2), tile point (x, y) of plane k, from
// the H ring (ring = plane k, ring ^ 1 = plane k-1); stA holds plane k
template <typename T, int GC, bool CHECK>
__device__ __forceinline__ void fused_e(const FusedCtx<T> &X, int x, int y, int k, int stA, int ring, bool pml_plane,
                                        bool slots, bool dft)
{
    using SH = FusedShape<T>;
    constexpr int BX = SH::BX, XOFF = SH::XOFF, c = GC;
    const FusedParams<T> &F = X.L->fp;
    const SideParams<T> &PE = F.e;
    if (CHECK && (x < PE.vlo[c][0] || x > PE.vhi[c][0] || y < PE.vlo[c][1] || y > PE.vhi[c][1] || k < PE.vlo[c][2] ||
                  k > PE.vhi[c][2]))
        return;
    const int row = y - (X.y0 - 1), col = x - (X.x0 - 1), prev = ring ^ 1;
    T curl1, curl2;
    if (c == 0)  // Ex: dHz/dy - dHy/dz
    {
        curl1 = (X.hn_at(ring, 2, row, col) - X.hn_at(ring, 2, row - 1, col)) * PE.inv_dx;
        curl2 = (X.hn_at(ring, 1, row, col) - X.hn_at(prev, 1, row, col)) * PE.inv_dx;
    }
    else if (c == 1)  // Ey: dHx/dz - dHz/dx
    {
        curl1 = (X.hn_at(ring, 0, row, col) - X.hn_at(prev, 0, row, col)) * PE.inv_dx;
        curl2 = (X.hn_at(ring, 2, row, col) - X.hn_at(ring, 2, row, col - 1)) * PE.inv_dx;
    }
    else  // Ez: dHy/dx - dHx/dy
    {
        curl1 = (X.hn_at(ring, 1, row, col) - X.hn_at(ring, 1, row, col - 1)) * PE.inv_dx;
        curl2 = (X.hn_at(ring, 0, row, col) - X.hn_at(ring, 0, row - 1, col)) * PE.inv_dx;
    }
    const int idx = x + y * (int)PE.sy + k * (int)PE.sz;
    const T term = fused_term<T, GC>(X, pml_plane, x, y, k, idx, curl1, curl2, PE.psi[c][0], PE.psi[c][1], PE.psi[c][0],
                                     PE.psi[c][1]);
    const T old = X.e_tile(stA, c)[(y - (X.y0 - 1)) * BX + (x - (X.x0 - XOFF))];
    T v, vd;
    if (!slots)
    {
        v = old + PE.coef_def * term;
        vd = PE.g_def * v;
    }
    else
        v = material_at(PE, PE.slot[c], slot_of(PE.slot[c], PE.My, x, y, k, idx), old, term, &vd);
    F.eout[c][idx] = v;
    if (dft) dft_point<T>(PE.nunits, PE.units, PE.phase, GC, x, y, k, (double)v, (double)vd);
}

template <typename T>
__global__ void __launch_bounds__(256, FusedShape<T>::MINB) k_fused(const __grid_constant__ FusedLaunch<T> L)
{
    using SH = FusedShape<T>;
    using LY = FusedLayout<T>;
    constexpr int TX = SH::TX, TY = SH::TY, XOFF = SH::XOFF, S = SH::S, KCH = SH::KCH;
    extern __shared__ __align__(128) unsigned char smem[];
    const FusedParams<T> &F = L.fp;
    const SideParams<T> &PE = F.e;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    FusedCtx<T> X;
    X.smem = smem;
    X.L = &L;
    X.x0 = blockIdx.x * TX;
    X.y0 = blockIdx.y * TY;
    X.k0 = blockIdx.z * KCH;
    const int k1 = min(X.k0 + KCH, PE.Mz);
    const int NP = k1 - X.k0 + 2;  // planes k0-1 .. k1
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    volatile int *flag = reinterpret_cast<volatile int *>(smem + 64);

    if (tid == 0)
    {
        for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int p) {
        const int st = p % S, z = X.k0 - 1 + p;
        mbar_expect_tx(&bar[st], LY::TX_BYTES);
        unsigned char *base = smem + 128 + st * LY::STAGE;
        for (int c = 0; c < 3; ++c) tma_load_3d(base + c * LY::E_TILE, &L.tm_e[c], X.x0 - XOFF, X.y0 - 1, z, &bar[st]);
        for (int c = 0; c < 3; ++c)
            tma_load_3d(base + 3 * LY::E_TILE + c * LY::H_TILE, &L.tm_h[c], X.x0 - XOFF, X.y0 - 1, z, &bar[st]);
    };
    int issued = min(S, NP);
    if (tid == 0)
        for (int p = 0; p < issued; ++p) issue(p);

    // stage the CPML tables of this tile / chunk while the first planes load
    const bool pml_tables = PE.pc[0][0] != nullptr;
    bool tile_pml = false;
    if (pml_tables)
    {
        for (int a = 0; a < 3; ++a)
        {
            const int n = a == 0 ? LY::NX : a == 1 ? LY::NY : LY::NZ;
            const int first = a == 0 ? X.x0 - 1 : a == 1 ? X.y0 - 1 : X.k0 - 1;
            const int len = a == 0 ? PE.Mx : a == 1 ? PE.My : PE.Mz;
            T *tab = X.pml(a);
            for (int t = tid; t < 2 * n; t += TX * TY)
            {
                const int q = t / n, o = t % n, pos = first + o;
                const bool in = pos >= 0 && pos < len;
                const T cv = in ? PE.pc[a][q][pos] : T(0);
                tab[(q * 3 + 0) * n + o] = in ? PE.pb[a][q][pos] : T(0);
                tab[(q * 3 + 1) * n + o] = cv;
                tab[(q * 3 + 2) * n + o] = in ? PE.pik[a][q][pos] : T(1);
                if (a < 2 && cv != T(0)) tile_pml = true;
            }
        }
    }
    // per plane of the chunk, which tile rows contain E-side material slots in
    // the tile's x range (one batch of loads, while the first planes arrive)
    unsigned *slot_mask = reinterpret_cast<unsigned *>(smem + LY::MASK_OFF);
    for (int t = tid; t < LY::NZ; t += TX * TY) slot_mask[t] = 0u;
    __syncthreads();
    for (int t = tid; t < LY::NZ * TY * 3; t += TX * TY)
    {
        const int c = t % 3, r = (t / 3) % TY, o = t / (3 * TY);
        const int kk = X.k0 - 1 + o, yy = X.y0 + r;
        if (!PE.slot[c].map || kk < 0 || kk >= PE.Mz || yy >= PE.My) continue;
        const RowRange rr = PE.slot[c].rows[yy + (int64_t)kk * PE.My];
        if (rr.lo <= rr.hi && rr.lo < X.x0 + TX && rr.hi >= X.x0) atomicOr(&slot_mask[o], 1u << r);
    }
    tile_pml = __syncthreads_or(tile_pml);
    // the tile and its low-side halo lie inside every component's valid x/y
    // range; kin_lo..kin_hi: planes where every component is valid
    bool tile_inside = true;
    int kin_lo = 0, kin_hi = PE.Mz;
    for (int sd = 0; sd < 2; ++sd)
    {
        const SideParams<T> &P = sd == 0 ? PE : F.h;
        for (int c = 0; c < 3; ++c)
        {
            tile_inside = tile_inside && P.vlo[c][0] <= X.x0 - 1 && X.x0 + TX - 1 <= P.vhi[c][0] && P.vlo[c][1] <= X.y0 - 1 &&
                          X.y0 + TY - 1 <= P.vhi[c][1];
            kin_lo = max(kin_lo, P.vlo[c][2]);
            kin_hi = min(kin_hi, P.vhi[c][2]);
        }
    }
    const bool h_slots = F.h.slot[0].map || F.h.slot[1].map || F.h.slot[2].map;

    const int x = X.x0 + tx, y = X.y0 + ty;
    // per-thread constants of the vacuum path
    constexpr int BX = SH::BX;
    const int offE = (ty + 1) * BX + tx + XOFF;  // own point in an E or H stage tile
    const int offN = (ty + 1) * (TX + 1) + tx + 1;  // own point in an H ring plane
    const int sz = (int)PE.sz;
    const int own0 = x + y * (int)PE.sy;
    const T coefH = F.h.coef_def, coefE = PE.coef_def, idh = F.h.inv_dx, ide = PE.inv_dx;
    for (int q = 0; q + 1 < NP; ++q)
    {
        const int stA = q % S, stB = (q + 1) % S;
        if (tid == 0)
        {
            bool ok = true;
            if (q == 0) ok = mbar_wait_bounded(&bar[stA], 0);
            ok = ok && mbar_wait_bounded(&bar[stB], ((q + 1) / S) & 1);
            *flag = ok ? 1 : 0;
        }
        __syncthreads();
        if (!*flag)
        {
            if (tid == 0)
            {
                atomicExch(L.err, 1);
                for (int p = q; p < issued; ++p) mbar_wait_bounded(&bar[p % S], (p / S) & 1);
            }
            return;
        }
        // every thread is past plane q-1, so its stage can be refilled
        if (tid == 0 && q >= 1 && q - 1 + S < NP)
        {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(q - 1 + S);
            issued = q + S;
        }
        const int k = X.k0 - 1 + q;
        const bool owned = q >= 1;
        const int ring = q & 1;
        bool pml_plane = false;
        if (pml_tables)
            pml_plane = tile_pml || X.template pml_val<2>(0, 1, k) != T(0) || X.template pml_val<2>(1, 1, k) != T(0);
        // CTA-uniform: every point of the tile (and its halo) valid in every
        // component at this plane?
        const bool inside = tile_inside && k >= kin_lo && k <= kin_hi;
        // DFT units touching this tile plane (E and H sides)
        bool dft_e = false, dft_h = false;
        for (int u = 0; u < PE.nunits; ++u)
        {
            const DftView &U = PE.units[u];
            dft_e = dft_e || (k >= U.i0[2] && k < U.i0[2] + U.ld[2] && U.i0[1] < X.y0 + TY && U.i0[1] + U.ld[1] > X.y0 &&
                              U.i0[0] < X.x0 + TX && U.i0[0] + U.ld[0] > X.x0);
        }
        for (int u = 0; u < F.h.nunits; ++u)
        {
            const DftView &U = F.h.units[u];
            dft_h = dft_h || (k >= U.i0[2] && k < U.i0[2] + U.ld[2] && U.i0[1] < X.y0 + TY && U.i0[1] + U.ld[1] > X.y0 &&
                              U.i0[0] < X.x0 + TX && U.i0[0] + U.ld[0] > X.x0);
        }
        const bool h_fast = inside && !pml_plane && !h_slots && !dft_h;
        if (h_fast)
        {
            // 1a. vacuum tile plane: H(k) from 12 staged values, no branches
            const T *eA0 = X.e_tile(stA, 0), *eA1 = X.e_tile(stA, 1), *eA2 = X.e_tile(stA, 2);
            const T *eB0 = X.e_tile(stB, 0), *eB1 = X.e_tile(stB, 1);
            const T *hA0 = X.h_tile(stA, 0), *hA1 = X.h_tile(stA, 1), *hA2 = X.h_tile(stA, 2);
            const T exa = eA0[offE], exy = eA0[offE + BX], exb = eB0[offE];
            const T eya = eA1[offE], eyx = eA1[offE + 1], eyb = eB1[offE];
            const T eza = eA2[offE], ezy = eA2[offE + BX], ezx = eA2[offE + 1];
            const T hx0 = hA0[offE], hy0 = hA1[offE], hz0 = hA2[offE];
            const T hx = hx0 + coefH * ((eza - ezy) * idh - (eya - eyb) * idh);
            const T hy = hy0 + coefH * ((exa - exb) * idh - (eza - ezx) * idh);
            const T hz = hz0 + coefH * ((eya - eyx) * idh - (exa - exy) * idh);
            X.hn_at(ring, 0, ty + 1, tx + 1) = hx;
            X.hn_at(ring, 1, ty + 1, tx + 1) = hy;
            X.hn_at(ring, 2, ty + 1, tx + 1) = hz;
            if (owned)
            {
                const int idx = own0 + k * sz;
                F.hout[0][idx] = hx;
                F.hout[1][idx] = hy;
                F.hout[2][idx] = hz;
            }
            // halo: Hz, Hx on the low-y row (row 0), Hz, Hy on the low-x column
            if (tid < 2 * TX + 2 * TY)
            {
                if (tid < 2 * TX)
                {
                    const int u = tid < TX ? tid : tid - TX, o = u + XOFF;  // row 0 of the tiles
                    if (tid < TX)
                        X.hn_at(ring, 2, 0, u + 1) = hA2[o] + coefH * ((eA1[o] - eA1[o + 1]) * idh - (eA0[o] - eA0[o + BX]) * idh);
                    else
                        X.hn_at(ring, 0, 0, u + 1) = hA0[o] + coefH * ((eA2[o] - eA2[o + BX]) * idh - (eA1[o] - eB1[o]) * idh);
                }
                else
                {
                    const int v = tid < 2 * TX + TY ? tid - 2 * TX : tid - 2 * TX - TY;
                    const int o = (v + 1) * BX + XOFF - 1;  // column x0 - 1
                    if (tid < 2 * TX + TY)
                        X.hn_at(ring, 2, v + 1, 0) = hA2[o] + coefH * ((eA1[o] - eA1[o + 1]) * idh - (eA0[o] - eA0[o + BX]) * idh);
                    else
                        X.hn_at(ring, 1, v + 1, 0) = hA1[o] + coefH * ((eA0[o] - eB0[o]) * idh - (eA2[o] - eA2[o + 1]) * idh);
                }
            }
        }
        else
        {
            // 1b. general tile plane: H(k) on the tile ...
            X.hn_at(ring, 0, ty + 1, tx + 1) = fused_h<T, 3, true>(X, x, y, k, stA, stB, owned, pml_plane, h_slots, dft_h);
            X.hn_at(ring, 1, ty + 1, tx + 1) = fused_h<T, 4, true>(X, x, y, k, stA, stB, owned, pml_plane, h_slots, dft_h);
            X.hn_at(ring, 2, ty + 1, tx + 1) = fused_h<T, 5, true>(X, x, y, k, stA, stB, owned, pml_plane, h_slots, dft_h);
            // ... and the halo the E update reads (recomputed, not written)
            if (tid < 2 * TX + 2 * TY)
            {
                int hx, hy, comp, row, col;
                if (tid < TX) { hx = X.x0 + tid; hy = X.y0 - 1; comp = 2; row = 0; col = tid + 1; }
                else if (tid < 2 * TX) { hx = X.x0 + tid - TX; hy = X.y0 - 1; comp = 0; row = 0; col = tid - TX + 1; }
                else if (tid < 2 * TX + TY) { hx = X.x0 - 1; hy = X.y0 + tid - 2 * TX; comp = 2; row = tid - 2 * TX + 1; col = 0; }
                else { hx = X.x0 - 1; hy = X.y0 + tid - 2 * TX - TY; comp = 1; row = tid - 2 * TX - TY + 1; col = 0; }
                T v = T(0);
                if (hx >= 0 && hy >= 0)
                {
                    if (comp == 0) v = fused_h<T, 3, true>(X, hx, hy, k, stA, stB, false, pml_plane, h_slots, false);
                    else if (comp == 1) v = fused_h<T, 4, true>(X, hx, hy, k, stA, stB, false, pml_plane, h_slots, false);
                    else v = fused_h<T, 5, true>(X, hx, hy, k, stA, stB, false, pml_plane, h_slots, false);
                }
                X.hn_at(ring, comp, row, col) = v;
            }
        }
        // material slots of the E components in this warp's row (warp-uniform)
        const bool e_slots = (slot_mask[q] >> ty) & 1u;
        __syncthreads();
        // 2. E(k) on the tile from H(k) and H(k-1)
        if (owned)
        {
            if (inside && !pml_plane && !e_slots && !dft_e)
            {
                const int prev = ring ^ 1;
                const T *eA0 = X.e_tile(stA, 0), *eA1 = X.e_tile(stA, 1), *eA2 = X.e_tile(stA, 2);
                const T *n0 = &X.hn_at(ring, 0, 0, 0), *n1 = &X.hn_at(ring, 1, 0, 0), *n2 = &X.hn_at(ring, 2, 0, 0);
                const T *p0 = &X.hn_at(prev, 0, 0, 0), *p1 = &X.hn_at(prev, 1, 0, 0);
                const T hzr = n2[offN], hzy = n2[offN - (TX + 1)], hzx = n2[offN - 1];
                const T hyr = n1[offN], hyp = p1[offN], hyx = n1[offN - 1];
                const T hxr = n0[offN], hxp = p0[offN], hxy = n0[offN - (TX + 1)];
                const T ex0 = eA0[offE], ey0 = eA1[offE], ez0 = eA2[offE];
                const T ex = ex0 + coefE * ((hzr - hzy) * ide - (hyr - hyp) * ide);
                const T ey = ey0 + coefE * ((hxr - hxp) * ide - (hzr - hzx) * ide);
                const T ez = ez0 + coefE * ((hyr - hyx) * ide - (hxr - hxy) * ide);
                const int idx = own0 + k * sz;
                F.eout[0][idx] = ex;
                F.eout[1][idx] = ey;
                F.eout[2][idx] = ez;
            }
            else
            {
                fused_e<T, 0, true>(X, x, y, k, stA, ring, pml_plane, e_slots, dft_e);
                fused_e<T, 1, true>(X, x, y, k, stA, ring, pml_plane, e_slots, dft_e);
                fused_e<T, 2, true>(X, x, y, k, stA, ring, pml_plane, e_slots, dft_e);
            }
        }
    }
}
} // namespace ffipg
