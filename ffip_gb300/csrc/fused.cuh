// Fused H+E time step: one z-marching pass over the grid per time step.
//
// Each CTA owns a TX x TY tile in (x, y), starting at index 1 (the first
// index that holds grid points), and marches a chunk of z planes (the valid z
// range split evenly over the grid's z blocks).  Iteration q of the march
// computes H at plane k = k0 - 1 + q and E at plane k - 1:
//   H(k) needs E(k), E(k+1) and H(k) of the previous level, staged in shared
//   memory by TMA (cp.async.bulk.tensor, one 3-D tensor map per field array)
//   through two rings completed by mbarriers: E planes (box TY + 2 rows, also
//   the E values of the E update one iteration later) and H planes (box
//   TY + 1 rows).  The new H goes into a three-plane ring in shared memory,
//   on the tile and on the low-x column and low-y row that the tile's E
//   update needs (those halo points belong to neighbouring CTAs and are
//   recomputed here, not written).
//   E(k-1) needs H(k-1) and H(k-2) from that ring, both completed in earlier
//   iterations, so one block barrier per iteration orders everything: H(k)
//   writes one ring plane while E(k-1) reads the other two.
// Every field value is read from HBM once and written once per time step.
// Because neighbouring CTAs read the previous level while this CTA writes the
// new one, field buffers (and the H-side CPML psi) ping-pong between steps;
// E-side CPML psi and polarisation state are only touched by their owner and
// are updated in place.  Each chunk starts by recomputing H of the plane
// below it (no writes).  Used with "None" boundaries on every face and no
// magnetic poles (the engine checks this).
//
// Two code paths per side and plane.  The common one (a tile plane with no
// CPML, no material slot, no DFT unit, every point valid) is the plain curl
// update.  The general one gates stores by per-thread validity bits (one per
// component), takes the CPML coefficients from per-axis tables staged in
// shared memory (E components use only parity-0 positions along their curl
// axes and H components only parity-1 positions, so one (b, c, 1/k) triple
// per axis and side) and handles material slots and DFT sums; its psi values
// are loaded at the top of the iteration, before the TMA wait.  The choice
// is CTA-uniform (warp-uniform for E material slots) and comes from flags
// precomputed once per CTA.
//
// When the valid x (y) extent exceeds a whole number of tiles by one or two
// points, those last layers are left to k_face (two small launches after this
// pass: H then E), so that no CTA is spent on a nearly empty tile.
//
// The per-point arithmetic is the same as the separate H/E kernels
// (stencil.cuh: pml_term, material_at, dft_point), so both passes give the
// same bits.  Only thread 0 waits on the mbarriers (bounded); on a timeout it
// records an error word, waits (bounded) for its outstanding copies, and the
// whole CTA returns.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.hpp"

namespace ffipg
{
template <typename T>
struct FusedShape;
// SE / SH: TMA stages of the E / H plane rings; KCH: most z planes per CTA;
// MINB: CTAs per SM the register budget is sized for (tuning builds may
// override the defaults).  Tiles start at x0 = 1 + TX * bx, so the TMA box
// starts at x0 - XOFF, a 16-byte boundary, and spans BX >= XOFF + TX + 1
// elements (x0 - 1 .. x0 + TX are needed).
#ifndef FFIP_FUSED_F32_SE
#define FFIP_FUSED_F32_SE 5
#endif
#ifndef FFIP_FUSED_F32_SH
#define FFIP_FUSED_F32_SH 3
#endif
#ifndef FFIP_FUSED_F32_MINB
#define FFIP_FUSED_F32_MINB 3
#endif
#ifndef FFIP_FUSED_F64_SE
#define FFIP_FUSED_F64_SE 4
#endif
#ifndef FFIP_FUSED_F64_SH
#define FFIP_FUSED_F64_SH 3
#endif
#ifndef FFIP_FUSED_F64_MINB
#define FFIP_FUSED_F64_MINB 2
#endif
#ifndef FFIP_FUSED_KCH
#define FFIP_FUSED_KCH 16
#endif
template <>
struct FusedShape<float>
{
    static constexpr int TX = 32, TY = 8, XOFF = 5, BX = 40, SE = FFIP_FUSED_F32_SE, SH = FFIP_FUSED_F32_SH,
                         KCH = FFIP_FUSED_KCH, MINB = FFIP_FUSED_F32_MINB;
};
template <>
struct FusedShape<double>
{
    static constexpr int TX = 32, TY = 8, XOFF = 3, BX = 36, SE = FFIP_FUSED_F64_SE, SH = FFIP_FUSED_F64_SH,
                         KCH = FFIP_FUSED_KCH, MINB = FFIP_FUSED_F64_MINB;
};

// CPML coefficients of one position along one axis: b, c, 1/k
template <typename T>
struct alignas(4 * sizeof(T)) PmlCoef
{
    T b, c, ik, pad;
};

template <typename T>
struct FusedLayout
{
    using SH = FusedShape<T>;
    static constexpr int E_BYTES = (SH::TY + 2) * SH::BX * (int)sizeof(T);  // one E box
    static constexpr int H_BYTES = (SH::TY + 1) * SH::BX * (int)sizeof(T);  // one H box
    static constexpr int E_TILE = (E_BYTES + 127) / 128 * 128;
    static constexpr int H_TILE = (H_BYTES + 127) / 128 * 128;
    static constexpr int E_OFF = 128;  // [0, 128): mbarriers and the wait flag
    static constexpr int H_OFF = E_OFF + SH::SE * 3 * E_TILE;
    static constexpr int HN_OFF = H_OFF + SH::SH * 3 * H_TILE;
    static constexpr int HN_PLANE = 3 * (SH::TY + 1) * (SH::TX + 1);  // elements of one H ring plane
    static constexpr int NX = SH::TX + 1, NY = SH::TY + 1, NZ = SH::KCH + 2;  // CPML table lengths
    static constexpr int PML_OFF = (HN_OFF + 3 * HN_PLANE * (int)sizeof(T) + 31) / 32 * 32;
    static constexpr int PML_BYTES = 2 * (NX + NY + NZ) * (int)sizeof(PmlCoef<T>);  // [axis][parity][n]
    static constexpr int INFO_OFF = PML_OFF + PML_BYTES;
    static constexpr int SMEM = INFO_OFF + NZ * 4;
    static_assert((SH::SE + SH::SH) * 8 <= 120, "mbarriers do not fit");
    static_assert(SH::BX >= SH::XOFF + SH::TX + 1, "TMA box too narrow");
    static_assert((SH::XOFF - 1) * (int)sizeof(T) % 16 == 0, "TMA box start off a 16-byte boundary");
    static_assert(SH::BX * (int)sizeof(T) % 16 == 0, "TMA box width not a multiple of 16 bytes");
};

// per-plane flag word (one per plane of the chunk, shared memory)
constexpr unsigned kInfoZValidShift = 8;   // bits 8..13: component c valid at this z
constexpr unsigned kInfoZPml = 1u << 14;   // CPML along z at this plane (either parity)
constexpr unsigned kInfoDftE = 1u << 15;   // an E DFT unit meets this tile plane
constexpr unsigned kInfoDftH = 1u << 16;   // an H DFT unit meets this tile plane
constexpr unsigned kInfoFastH = 1u << 17;  // H of this tile plane takes the plain path
constexpr unsigned kInfoFastE = 1u << 18;  // E of this tile plane takes the plain path (rows without slots)
                                           // bits 0..TY-1: tile row r has E material slots

template <typename T>
struct FusedLaunch
{
    CUtensorMap tm_e[3];  // E input arrays, box (BX, TY + 2, 1)
    CUtensorMap tm_h[3];  // H input arrays, box (BX, TY + 1, 1)
    FusedParams<T> fp;
    int *err;             // set to 1 when a wait times out
    int xlim, ylim;       // this pass updates 1 <= x < xlim, 1 <= y < ylim; k_face the rest
    int xend, yend;       // valid extents (max over components of vhi + 1)
    int kbeg, kend;       // valid z range split over the grid's z blocks
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
    // E box of E stage st (rows y0-1 .. y0+TY), H box of H stage st (rows y0-1 .. y0+TY-1)
    __device__ __forceinline__ const T *e_tile(int st, int c) const
    {
        return reinterpret_cast<const T *>(smem + LY::E_OFF + (st * 3 + c) * LY::E_TILE);
    }
    __device__ __forceinline__ const T *h_tile(int st, int c) const
    {
        return reinterpret_cast<const T *>(smem + LY::H_OFF + (st * 3 + c) * LY::H_TILE);
    }
    // new H, ring plane r (0..2), rows y0-1 .. y0+TY-1, columns x0-1 .. x0+TX-1
    __device__ __forceinline__ T &hn_at(int r, int c, int row, int col) const
    {
        return reinterpret_cast<T *>(smem + LY::HN_OFF)[r * LY::HN_PLANE + (c * (SH::TY + 1) + row) * (SH::TX + 1) + col];
    }
    // CPML table of axis a, parity q: entry o is position first_a + o, with
    // first = x0 - 1, y0 - 1, k0 - 1
    __device__ __forceinline__ PmlCoef<T> *tab(int a, int q) const
    {
        PmlCoef<T> *base = reinterpret_cast<PmlCoef<T> *>(smem + LY::PML_OFF);
        return a == 0 ? base + q * LY::NX : a == 1 ? base + 2 * LY::NX + q * LY::NY : base + 2 * (LY::NX + LY::NY) + q * LY::NZ;
    }
    template <int A>
    __device__ __forceinline__ T pml_val(int q, int v, int pos) const
    {
        const int o = A == 0 ? pos - (x0 - 1) : A == 1 ? pos - (y0 - 1) : pos - (k0 - 1);
        const PmlCoef<T> &e = tab(A, q)[o];
        return v == 0 ? e.b : v == 1 ? e.c : e.ik;
    }
};

// accdb increment at one point of component GC from its two curls, CPML
// coefficients taken from the staged tables (halo points)
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

// H at the new level of a halo point (not owned: nothing is written),
// component GC (3..5), point (x, y) of plane k; E stages eA/eB hold planes
// k/k+1, H stage hA plane k.  Returns 0 where the component has no grid point.
template <typename T, int GC>
__device__ __forceinline__ T fused_h_halo(const FusedCtx<T> &X, int x, int y, int k, int eA, int eB, int hA, bool pml_plane,
                                          bool slots)
{
    using SH = FusedShape<T>;
    constexpr int BX = SH::BX, XOFF = SH::XOFF, c = GC - 3;
    const FusedParams<T> &F = X.L->fp;
    const SideParams<T> &PH = F.h;
    if (x < PH.vlo[c][0] || x > PH.vhi[c][0] || y < PH.vlo[c][1] || y > PH.vhi[c][1] || k < PH.vlo[c][2] ||
        k > PH.vhi[c][2])
        return T(0);
    const int o = (y - (X.y0 - 1)) * BX + x - (X.x0 - XOFF);
    T curl1, curl2;
    if (c == 0)  // Hx: -(dEz/dy) + dEy/dz
    {
        const T *Ez = X.e_tile(eA, 2), *Ey = X.e_tile(eA, 1);
        curl1 = (Ez[o] - Ez[o + BX]) * PH.inv_dx;
        curl2 = (Ey[o] - X.e_tile(eB, 1)[o]) * PH.inv_dx;
    }
    else if (c == 1)  // Hy: -(dEx/dz) + dEz/dx
    {
        const T *Ex = X.e_tile(eA, 0), *Ez = X.e_tile(eA, 2);
        curl1 = (Ex[o] - X.e_tile(eB, 0)[o]) * PH.inv_dx;
        curl2 = (Ez[o] - Ez[o + 1]) * PH.inv_dx;
    }
    else  // Hz: -(dEy/dx) + dEx/dy
    {
        const T *Ey = X.e_tile(eA, 1), *Ex = X.e_tile(eA, 0);
        curl1 = (Ey[o] - Ey[o + 1]) * PH.inv_dx;
        curl2 = (Ex[o] - Ex[o + BX]) * PH.inv_dx;
    }
    const int idx = x + y * (int)PH.sy + k * (int)PH.sz;
    const T term = fused_term<T, GC>(X, pml_plane, x, y, k, idx, curl1, curl2, F.psih_in[c][0], F.psih_in[c][1], nullptr,
                                     nullptr);
    const T old = X.h_tile(hA, c)[o];
    T vd;
    if (!slots) return old + PH.coef_def * term;
    return material_at(PH, PH.slot[c], slot_of(PH.slot[c], PH.My, x, y, k, idx), old, term, &vd);
}

// curl term of one component from its two curls with the CPML coefficients
// of its two curl axes (cv == 0 on both: plain curl, as Curl_Stepping)
template <typename T>
__device__ __forceinline__ T plane_term(const PmlCoef<T> &A1, const PmlCoef<T> &A2, T curl1, T curl2, T psi1, T psi2, T *ps1,
                                        T *ps2)
{
    if (A1.c == T(0) && A2.c == T(0)) return curl1 - curl2;
    return pml_term(A1.c, A2.c, A1.b, A2.b, A1.ik, A2.ik, curl1, curl2, psi1, psi2, ps1, ps2);
}

// General H(k) at this thread's own tile point: validity bits, CPML from the
// staged tables (psi values ph loaded by the caller), material slots, DFT.
template <typename T>
__device__ __forceinline__ void h_own_general(const FusedCtx<T> &X, int q, int eA, int eB, int hA, int slot_new, unsigned vb,
                                              bool owned, bool pml, bool slots, bool dft, int idx, const T (&ph)[3][2])
{
    using SH = FusedShape<T>;
    constexpr int BX = SH::BX;
    const FusedParams<T> &F = X.L->fp;
    const SideParams<T> &PH = F.h;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int offE = (ty + 1) * BX + tx + SH::XOFF;
    const T idh = PH.inv_dx;
    const T *eA0 = X.e_tile(eA, 0), *eA1 = X.e_tile(eA, 1), *eA2 = X.e_tile(eA, 2);
    const T *eB0 = X.e_tile(eB, 0), *eB1 = X.e_tile(eB, 1);
    const T exa = eA0[offE], exy = eA0[offE + BX], exb = eB0[offE];
    const T eya = eA1[offE], eyx = eA1[offE + 1], eyb = eB1[offE];
    const T eza = eA2[offE], ezy = eA2[offE + BX], ezx = eA2[offE + 1];
    T curl1[3], curl2[3];
    curl1[0] = (eza - ezy) * idh;  // Hx: -(dEz/dy) + dEy/dz
    curl2[0] = (eya - eyb) * idh;
    curl1[1] = (exa - exb) * idh;  // Hy: -(dEx/dz) + dEz/dx
    curl2[1] = (eza - ezx) * idh;
    curl1[2] = (eya - eyx) * idh;  // Hz: -(dEy/dx) + dEx/dy
    curl2[2] = (exa - exy) * idh;
    PmlCoef<T> hc[3] = {};  // per axis, parity 1
    if (pml)
    {
        hc[0] = X.tab(0, 1)[tx + 1];
        hc[1] = X.tab(1, 1)[ty + 1];
        hc[2] = X.tab(2, 1)[q];
    }
    const int x = X.x0 + tx, y = X.y0 + ty, k = X.k0 - 1 + q;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        T ps1 = T(0), ps2 = T(0);
        const T term = plane_term(hc[a1], hc[a2], curl1[c], curl2[c], ph[c][0], ph[c][1], &ps1, &ps2);
        const T old = X.h_tile(hA, c)[offE];
        T v, vd;
        if (!slots)
        {
            v = old + PH.coef_def * term;
            vd = PH.g_def * v;
        }
        else
            v = material_at(PH, PH.slot[c], slot_of(PH.slot[c], PH.My, x, y, k, idx), old, term, &vd);
        const bool val = (vb >> (3 + c)) & 1u;
        X.hn_at(slot_new, c, ty + 1, tx + 1) = val ? v : T(0);
        if (owned && val)
        {
            F.hout[c][idx] = v;
            if (hc[a1].c != T(0)) F.psih_out[c][0][idx] = ps1;
            if (hc[a2].c != T(0)) F.psih_out[c][1][idx] = ps2;
            if (dft) dft_point<T>(PH.nunits, PH.units, PH.phase, 3 + c, x, y, k, (double)v, (double)vd);
        }
    }
}

// General E(k) at this thread's own tile point (E plane qe of the chunk),
// from the H ring planes rn (plane k) and rp (plane k-1).
template <typename T>
__device__ __forceinline__ void e_own_general(const FusedCtx<T> &X, int qe, int eS, int rn, int rp, unsigned vb, bool pml,
                                              bool slots, bool dft, int idx, const T (&pe)[3][2], const int (&sl)[3])
{
    using SH = FusedShape<T>;
    constexpr int BX = SH::BX, TX = SH::TX;
    const FusedParams<T> &F = X.L->fp;
    const SideParams<T> &PE = F.e;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int offE = (ty + 1) * BX + tx + SH::XOFF;
    const int offN = (ty + 1) * (TX + 1) + tx + 1;
    PmlCoef<T> ec[3] = {};  // per axis, parity 0
    if (pml)
    {
        ec[0] = X.tab(0, 0)[tx + 1];
        ec[1] = X.tab(1, 0)[ty + 1];
        ec[2] = X.tab(2, 0)[qe];
    }
    const T ide = PE.inv_dx;
    const T *n0 = &X.hn_at(rn, 0, 0, 0), *n1 = &X.hn_at(rn, 1, 0, 0), *n2 = &X.hn_at(rn, 2, 0, 0);
    const T *p0 = &X.hn_at(rp, 0, 0, 0), *p1 = &X.hn_at(rp, 1, 0, 0);
    const T hzr = n2[offN], hzy = n2[offN - (TX + 1)], hzx = n2[offN - 1];
    const T hyr = n1[offN], hyp = p1[offN], hyx = n1[offN - 1];
    const T hxr = n0[offN], hxp = p0[offN], hxy = n0[offN - (TX + 1)];
    T curl1[3], curl2[3];
    curl1[0] = (hzr - hzy) * ide;  // Ex: dHz/dy - dHy/dz
    curl2[0] = (hyr - hyp) * ide;
    curl1[1] = (hxr - hxp) * ide;  // Ey: dHx/dz - dHz/dx
    curl2[1] = (hzr - hzx) * ide;
    curl1[2] = (hyr - hyx) * ide;  // Ez: dHy/dx - dHx/dy
    curl2[2] = (hxr - hxy) * ide;
    const int x = X.x0 + tx, y = X.y0 + ty, k = X.k0 - 1 + qe;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        T ps1 = T(0), ps2 = T(0);
        const T term = plane_term(ec[a1], ec[a2], curl1[c], curl2[c], pe[c][0], pe[c][1], &ps1, &ps2);
        const T old = X.e_tile(eS, c)[offE];
        T v, vd;
        if (!slots || sl[c] < 0)
        {
            v = old + PE.coef_def * term;
            vd = PE.g_def * v;
        }
        else
            v = material_rec(PE, PE.slot[c], sl[c], old, term, &vd);
        if ((vb >> c) & 1u)
        {
            F.eout[c][idx] = v;
            if (ec[a1].c != T(0)) PE.psi[c][0][idx] = ps1;
            if (ec[a2].c != T(0)) PE.psi[c][1][idx] = ps2;
            if (dft) dft_point<T>(PE.nunits, PE.units, PE.phase, c, x, y, k, (double)v, (double)vd);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256, FusedShape<T>::MINB) k_fused(const __grid_constant__ FusedLaunch<T> L)
{
    using SH = FusedShape<T>;
    using LY = FusedLayout<T>;
    constexpr int TX = SH::TX, TY = SH::TY, XOFF = SH::XOFF, SE = SH::SE, SHS = SH::SH, BX = SH::BX;
    extern __shared__ __align__(128) unsigned char smem[];
    const FusedParams<T> &F = L.fp;
    const SideParams<T> &PE = F.e;
    const SideParams<T> &PH = F.h;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    FusedCtx<T> X;
    X.smem = smem;
    X.L = &L;
    X.x0 = 1 + blockIdx.x * TX;
    X.y0 = 1 + blockIdx.y * TY;
    X.k0 = L.kbeg + (int)((int64_t)(L.kend - L.kbeg) * blockIdx.z / gridDim.z);
    const int k1 = L.kbeg + (int)((int64_t)(L.kend - L.kbeg) * (blockIdx.z + 1) / gridDim.z);
    const int NP = k1 - X.k0 + 2;  // planes k0-1 .. k1 (plane p is z = k0 - 1 + p)
    uint64_t *ebar = reinterpret_cast<uint64_t *>(smem);
    uint64_t *hbar = ebar + SE;
    volatile int *flag = reinterpret_cast<volatile int *>(smem + 120);

    if (tid == 0)
    {
        for (int s = 0; s < SE; ++s) mbar_init(&ebar[s], 1);
        for (int s = 0; s < SHS; ++s) mbar_init(&hbar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue_e = [&](int p) {
        const int st = p % SE;
        mbar_expect_tx(&ebar[st], 3 * LY::E_BYTES);
        for (int c = 0; c < 3; ++c)
            tma_load_3d(smem + LY::E_OFF + (st * 3 + c) * LY::E_TILE, &L.tm_e[c], X.x0 - XOFF, X.y0 - 1, X.k0 - 1 + p,
                        &ebar[st]);
    };
    auto issue_h = [&](int p) {
        const int st = p % SHS;
        mbar_expect_tx(&hbar[st], 3 * LY::H_BYTES);
        for (int c = 0; c < 3; ++c)
            tma_load_3d(smem + LY::H_OFF + (st * 3 + c) * LY::H_TILE, &L.tm_h[c], X.x0 - XOFF, X.y0 - 1, X.k0 - 1 + p,
                        &hbar[st]);
    };
    // E planes 0 .. NP-1 are used; H planes 0 .. NP-2
    int e_issued = min(SE, NP), h_issued = min(SHS, NP - 1);
    if (tid == 0)
    {
        for (int p = 0; p < e_issued; ++p) issue_e(p);
        for (int p = 0; p < h_issued; ++p) issue_h(p);
    }

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
            for (int t = tid; t < 2 * n; t += TX * TY)
            {
                const int q = t / n, o = t % n, pos = first + o;
                const bool in = pos >= 0 && pos < len;
                PmlCoef<T> e;
                e.b = in ? PE.pb[a][q][pos] : T(0);
                e.c = in ? PE.pc[a][q][pos] : T(0);
                e.ik = in ? PE.pik[a][q][pos] : T(1);
                e.pad = T(0);
                X.tab(a, q)[o] = e;
                if (a < 2 && e.c != T(0)) tile_pml = true;
            }
        }
    }
    // per plane of the chunk: flag word (z validity, z CPML, DFT units
    // meeting the tile plane, tile rows with E material slots)
    unsigned *info = reinterpret_cast<unsigned *>(smem + LY::INFO_OFF);
    for (int o = tid; o < LY::NZ; o += TX * TY)
    {
        const int k = X.k0 - 1 + o;
        unsigned w = 0;
        for (int c = 0; c < 3; ++c)
        {
            if (k >= PE.vlo[c][2] && k <= PE.vhi[c][2]) w |= 1u << (kInfoZValidShift + c);
            if (k >= PH.vlo[c][2] && k <= PH.vhi[c][2]) w |= 1u << (kInfoZValidShift + 3 + c);
        }
        if (pml_tables && k >= 0 && k < PE.Mz && (PE.pc[2][0][k] != T(0) || PE.pc[2][1][k] != T(0))) w |= kInfoZPml;
        for (int u = 0; u < PE.nunits; ++u)
        {
            const DftView &U = PE.units[u];
            if (k >= U.i0[2] && k < U.i0[2] + U.ld[2] && U.i0[1] < X.y0 + TY && U.i0[1] + U.ld[1] > X.y0 &&
                U.i0[0] < X.x0 + TX && U.i0[0] + U.ld[0] > X.x0)
                w |= kInfoDftE;
        }
        for (int u = 0; u < PH.nunits; ++u)
        {
            const DftView &U = PH.units[u];
            if (k >= U.i0[2] && k < U.i0[2] + U.ld[2] && U.i0[1] < X.y0 + TY && U.i0[1] + U.ld[1] > X.y0 &&
                U.i0[0] < X.x0 + TX && U.i0[0] + U.ld[0] > X.x0)
                w |= kInfoDftH;
        }
        info[o] = w;
    }
    __syncthreads();
    for (int t = tid; t < LY::NZ * TY * 3; t += TX * TY)
    {
        const int c = t % 3, r = (t / 3) % TY, o = t / (3 * TY);
        const int kk = X.k0 - 1 + o, yy = X.y0 + r;
        if (!PE.slot[c].map || kk < 0 || kk >= PE.Mz || yy >= PE.My) continue;
        const RowRange rr = PE.slot[c].rows[yy + (int64_t)kk * PE.My];
        if (rr.lo <= rr.hi && rr.lo < X.x0 + TX && rr.hi >= X.x0) atomicOr(&info[o], 1u << r);
    }
    tile_pml = __syncthreads_or(tile_pml);
    const bool h_slots = PH.slot[0].map || PH.slot[1].map || PH.slot[2].map;

    const int x = X.x0 + tx, y = X.y0 + ty;
    // components with a grid point at (x, y) that this pass owns
    unsigned vxy = 0;
    if (x < L.xlim && y < L.ylim)
        for (int c = 0; c < 3; ++c)
        {
            if (x >= PE.vlo[c][0] && x <= PE.vhi[c][0] && y >= PE.vlo[c][1] && y <= PE.vhi[c][1]) vxy |= 1u << c;
            if (x >= PH.vlo[c][0] && x <= PH.vhi[c][0] && y >= PH.vlo[c][1] && y <= PH.vhi[c][1]) vxy |= 1u << (3 + c);
        }
    // every own and halo point of the tile valid in x and y for all six components
    bool inside = X.x0 + TX <= L.xlim && X.y0 + TY <= L.ylim;
    for (int c = 0; c < 3; ++c)
        inside = inside && PE.vlo[c][0] <= X.x0 - 1 && X.x0 + TX - 1 <= PE.vhi[c][0] && PE.vlo[c][1] <= X.y0 - 1 &&
                 X.y0 + TY - 1 <= PE.vhi[c][1] && PH.vlo[c][0] <= X.x0 - 1 && X.x0 + TX - 1 <= PH.vhi[c][0] &&
                 PH.vlo[c][1] <= X.y0 - 1 && X.y0 + TY - 1 <= PH.vhi[c][1];
    // per plane: may each side take the plain path
    for (int o = tid; o < LY::NZ; o += TX * TY)
    {
        const unsigned w = info[o];
        const bool zpml = pml_tables && (tile_pml || (w & kInfoZPml));
        if (inside && !zpml && !h_slots && !(w & kInfoDftH) && ((w >> (kInfoZValidShift + 3)) & 7u) == 7u) info[o] |= kInfoFastH;
        if (inside && !zpml && !(w & kInfoDftE) && ((w >> kInfoZValidShift) & 7u) == 7u) info[o] |= kInfoFastE;
    }
    __syncthreads();
    const int sz = (int)PE.sz;
    const int own0 = x + y * (int)PE.sy;
    const int offE = (ty + 1) * BX + tx + XOFF;     // own point in an E or H box
    const int offN = (ty + 1) * (TX + 1) + tx + 1;  // own point in an H ring plane
    const T coefH = PH.coef_def, coefE = PE.coef_def, idh = PH.inv_dx, ide = PE.inv_dx;

    // material slot indices of the E plane of the next iteration, loaded one
    // iteration ahead (rows flagged in the plane word only)
    int sl_next[3] = {-1, -1, -1};
    // iteration q: H at plane k = k0 - 1 + q (q <= NP - 2), E at plane k - 1 (q >= 2)
    // running ring positions: E stages of planes q-1, q, q+1; H stage of
    // plane q; H ring planes of H(k), H(k-1), H(k-2)
    int eS = SE - 1, eA = 0, eB = 1 % SE, hA = 0, rn = 0, rp = 2, rpp = 1;
    int idx = own0 + (X.k0 - 1) * sz;
    for (int q = 0; q < NP; ++q, idx += sz)
    {
        const int sl_e[3] = {sl_next[0], sl_next[1], sl_next[2]};
        const bool do_h = q <= NP - 2, do_e = q >= 2;
        const int k = X.k0 - 1 + q;
        const int idx_e = idx - sz;
        const unsigned wh = info[q], we = q >= 1 ? info[q - 1] : 0u;
        const bool e_slots = (we >> ty) & 1u;
        const bool fast_h = wh & kInfoFastH;
        const bool fast_e = (we & kInfoFastE) && !e_slots;
        const unsigned vbh = vxy & (wh >> kInfoZValidShift), vbe = vxy & (we >> kInfoZValidShift);
        const bool pml_h = !fast_h && pml_tables && (tile_pml || (wh & kInfoZPml));
        const bool pml_e = !fast_e && pml_tables && (tile_pml || (we & kInfoZPml));
        const bool dft_h = wh & kInfoDftH, dft_e = we & kInfoDftE;
        // CPML psi of this iteration's own points, loaded before the TMA wait
        T ph[3][2] = {}, pe[3][2] = {};
        if (do_h && pml_h)
        {
            const T ch[3] = {X.tab(0, 1)[tx + 1].c, X.tab(1, 1)[ty + 1].c, X.tab(2, 1)[q].c};  // H side (parity 1)
#pragma unroll
            for (int c = 0; c < 3; ++c)
            {
                const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
                const bool vh = (vbh >> (3 + c)) & 1u;
                if (vh && ch[a1] != T(0)) ph[c][0] = F.psih_in[c][0][idx];
                if (vh && ch[a2] != T(0)) ph[c][1] = F.psih_in[c][1][idx];
            }
        }
        if (do_e && pml_e)
        {
            const T ce[3] = {X.tab(0, 0)[tx + 1].c, X.tab(1, 0)[ty + 1].c, X.tab(2, 0)[q - 1].c};  // E side (parity 0)
#pragma unroll
            for (int c = 0; c < 3; ++c)
            {
                const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
                const bool ve = (vbe >> c) & 1u;
                if (ve && ce[a1] != T(0)) pe[c][0] = PE.psi[c][0][idx_e];
                if (ve && ce[a2] != T(0)) pe[c][1] = PE.psi[c][1][idx_e];
            }
        }
        sl_next[0] = sl_next[1] = sl_next[2] = -1;
        if (q >= 1 && q <= NP - 2 && ((wh >> ty) & 1u))
        {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                if (PE.slot[c].map && ((vbh >> c) & 1u)) sl_next[c] = PE.slot[c].map[idx];
        }
        if (tid == 0)
        {
            bool ok = true;
            if (q == 0) ok = mbar_wait_bounded(&ebar[0], 0);
            if (q + 1 < NP) ok = ok && mbar_wait_bounded(&ebar[(q + 1) % SE], ((q + 1) / SE) & 1);
            if (do_h) ok = ok && mbar_wait_bounded(&hbar[q % SHS], (q / SHS) & 1);
            *flag = ok ? 1 : 0;
        }
        // (A): the planes are visible, and every thread is done with
        // iteration q-1 (ring plane q % 3 is free, E plane q-2 and H plane
        // q-1 can be refilled)
        __syncthreads();
        if (!*flag)
        {
            if (tid == 0)
            {
                atomicExch(L.err, 1);
                for (int p = 0; p < e_issued; ++p) mbar_wait_bounded(&ebar[p % SE], (p / SE) & 1);
                for (int p = 0; p < h_issued; ++p) mbar_wait_bounded(&hbar[p % SHS], (p / SHS) & 1);
            }
            return;
        }
        if (tid == 0)
        {
            bool fence = false;
            if (q >= 2 && q - 2 + SE < NP)
            {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                fence = true;
                issue_e(q - 2 + SE);
                e_issued = q - 1 + SE;
            }
            if (q >= 1 && q - 1 + SHS <= NP - 2)
            {
                if (!fence) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_h(q - 1 + SHS);
                h_issued = q + SHS;
            }
        }
        // 1. H(k) at the tile's own points, and the halo the E update of the
        //    next iteration reads: Hz, Hx on the low-y row, Hz, Hy on the
        //    low-x column (recomputed, not written)
        if (do_h)
        {
            if (fast_h)
            {
                const T *eA0 = X.e_tile(eA, 0), *eA1 = X.e_tile(eA, 1), *eA2 = X.e_tile(eA, 2);
                const T *eB0 = X.e_tile(eB, 0), *eB1 = X.e_tile(eB, 1);
                const T *hA0 = X.h_tile(hA, 0), *hA1 = X.h_tile(hA, 1), *hA2 = X.h_tile(hA, 2);
                const T exa = eA0[offE], exy = eA0[offE + BX], exb = eB0[offE];
                const T eya = eA1[offE], eyx = eA1[offE + 1], eyb = eB1[offE];
                const T eza = eA2[offE], ezy = eA2[offE + BX], ezx = eA2[offE + 1];
                const T hx = hA0[offE] + coefH * ((eza - ezy) * idh - (eya - eyb) * idh);
                const T hy = hA1[offE] + coefH * ((exa - exb) * idh - (eza - ezx) * idh);
                const T hz = hA2[offE] + coefH * ((eya - eyx) * idh - (exa - exy) * idh);
                X.hn_at(rn, 0, ty + 1, tx + 1) = hx;
                X.hn_at(rn, 1, ty + 1, tx + 1) = hy;
                X.hn_at(rn, 2, ty + 1, tx + 1) = hz;
                if (q >= 1)
                {
                    F.hout[0][idx] = hx;
                    F.hout[1][idx] = hy;
                    F.hout[2][idx] = hz;
                }
                if (tid < 2 * TX + 2 * TY)
                {
                    if (tid < 2 * TX)
                    {
                        const int u = tid < TX ? tid : tid - TX, o = u + XOFF;  // row y0 - 1 of the boxes
                        if (tid < TX)
                            X.hn_at(rn, 2, 0, u + 1) = hA2[o] + coefH * ((eA1[o] - eA1[o + 1]) * idh - (eA0[o] - eA0[o + BX]) * idh);
                        else
                            X.hn_at(rn, 0, 0, u + 1) = hA0[o] + coefH * ((eA2[o] - eA2[o + BX]) * idh - (eA1[o] - eB1[o]) * idh);
                    }
                    else
                    {
                        const int v = tid < 2 * TX + TY ? tid - 2 * TX : tid - 2 * TX - TY;
                        const int o = (v + 1) * BX + XOFF - 1;  // column x0 - 1
                        if (tid < 2 * TX + TY)
                            X.hn_at(rn, 2, v + 1, 0) = hA2[o] + coefH * ((eA1[o] - eA1[o + 1]) * idh - (eA0[o] - eA0[o + BX]) * idh);
                        else
                            X.hn_at(rn, 1, v + 1, 0) = hA1[o] + coefH * ((eA0[o] - eB0[o]) * idh - (eA2[o] - eA2[o + 1]) * idh);
                    }
                }
            }
            else
            {
                h_own_general<T>(X, q, eA, eB, hA, rn, vbh, q >= 1, pml_h, h_slots, dft_h, idx, ph);
                if (tid < 2 * TX + 2 * TY)
                {
                    int hx, hy, comp, row, col;
                    if (tid < TX) { hx = X.x0 + tid; hy = X.y0 - 1; comp = 2; row = 0; col = tid + 1; }
                    else if (tid < 2 * TX) { hx = X.x0 + tid - TX; hy = X.y0 - 1; comp = 0; row = 0; col = tid - TX + 1; }
                    else if (tid < 2 * TX + TY) { hx = X.x0 - 1; hy = X.y0 + tid - 2 * TX; comp = 2; row = tid - 2 * TX + 1; col = 0; }
                    else { hx = X.x0 - 1; hy = X.y0 + tid - 2 * TX - TY; comp = 1; row = tid - 2 * TX - TY + 1; col = 0; }
                    T v;
                    if (comp == 0) v = fused_h_halo<T, 3>(X, hx, hy, k, eA, eB, hA, pml_h, h_slots);
                    else if (comp == 1) v = fused_h_halo<T, 4>(X, hx, hy, k, eA, eB, hA, pml_h, h_slots);
                    else v = fused_h_halo<T, 5>(X, hx, hy, k, eA, eB, hA, pml_h, h_slots);
                    X.hn_at(rn, comp, row, col) = v;
                }
            }
        }
        // 2. E(k-1) on the tile from H(k-1) and H(k-2)
        if (do_e)
        {
            if (fast_e)
            {
                const T *eS0 = X.e_tile(eS, 0), *eS1 = X.e_tile(eS, 1), *eS2 = X.e_tile(eS, 2);
                const T *n0 = &X.hn_at(rp, 0, 0, 0), *n1 = &X.hn_at(rp, 1, 0, 0), *n2 = &X.hn_at(rp, 2, 0, 0);
                const T *p0 = &X.hn_at(rpp, 0, 0, 0), *p1 = &X.hn_at(rpp, 1, 0, 0);
                const T hzr = n2[offN], hzy = n2[offN - (TX + 1)], hzx = n2[offN - 1];
                const T hyr = n1[offN], hyp = p1[offN], hyx = n1[offN - 1];
                const T hxr = n0[offN], hxp = p0[offN], hxy = n0[offN - (TX + 1)];
                const T ex = eS0[offE] + coefE * ((hzr - hzy) * ide - (hyr - hyp) * ide);
                const T ey = eS1[offE] + coefE * ((hxr - hxp) * ide - (hzr - hzx) * ide);
                const T ez = eS2[offE] + coefE * ((hyr - hyx) * ide - (hxr - hxy) * ide);
                F.eout[0][idx_e] = ex;
                F.eout[1][idx_e] = ey;
                F.eout[2][idx_e] = ez;
            }
            else
                e_own_general<T>(X, q - 1, eS, rp, rpp, vbe, pml_e, e_slots, dft_e, idx_e, pe, sl_e);
        }
        eS = eA;
        eA = eB;
        eB = eB + 1 == SE ? 0 : eB + 1;
        hA = hA + 1 == SHS ? 0 : hA + 1;
        rpp = rp;
        rp = rn;
        rn = rn == 2 ? 0 : rn + 1;
    }
}

// One point of the last x / y layers that the fused pass leaves out (same
// update as update_point, with the fused pass's input/output buffers): H
// reads E and H at step n from the input buffers and writes the output
// buffers; E reads the new H from the output buffers.
template <typename T, int GC>
__device__ __forceinline__ void face_point(const FusedParams<T> &F, int i, int j, int k)
{
    using C = CompT<GC>;
    constexpr bool IS_E = GC < 3;
    constexpr int c = C::c;
    const SideParams<T> &p = IS_E ? F.e : F.h;
    const int64_t idx = (int64_t)i + (int64_t)j * p.sy + (int64_t)k * p.sz;
    const int64_t s1 = C::a1 == 0 ? 1 : (C::a1 == 1 ? p.sy : p.sz);
    const int64_t s2 = C::a2 == 0 ? 1 : (C::a2 == 1 ? p.sy : p.sz);
    const T *O1 = IS_E ? F.hout[C::a2] : F.ein[C::a2];
    const T *O2 = IS_E ? F.hout[C::a1] : F.ein[C::a1];
    T curl1, curl2;
    if (IS_E)
    {
        curl1 = (O1[idx] - O1[idx - s1]) * p.inv_dx;
        curl2 = (O2[idx] - O2[idx - s2]) * p.inv_dx;
    }
    else
    {
        curl1 = (O1[idx] - O1[idx + s1]) * p.inv_dx;
        curl2 = (O2[idx] - O2[idx + s2]) * p.inv_dx;
    }
    const T *pin1 = IS_E ? p.psi[c][0] : F.psih_in[c][0], *pin2 = IS_E ? p.psi[c][1] : F.psih_in[c][1];
    T *pout1 = IS_E ? p.psi[c][0] : F.psih_out[c][0], *pout2 = IS_E ? p.psi[c][1] : F.psih_out[c][1];
    const T term = curl_term_global<T, GC>(p, i, j, k, idx, curl1, curl2, pin1, pin2, pout1, pout2);
    const int slot = slot_of(p.slot[c], p.My, i, j, k, idx);
    const T old = IS_E ? F.ein[c][idx] : F.hin[c][idx];
    T vd;
    const T v = material_at(p, p.slot[c], slot, old, term, &vd);
    (IS_E ? F.eout : F.hout)[c][idx] = v;
    if (p.nunits) dft_point<T>(p.nunits, p.units, p.phase, GC, i, j, k, (double)v, (double)vd);
}

// The points with x >= xlim (all y) or y >= ylim (x < xlim), all z
template <typename T, bool IS_E>
__global__ void k_face(const __grid_constant__ FusedLaunch<T> L)
{
    const FusedParams<T> &F = L.fp;
    const SideParams<T> &p = IS_E ? F.e : F.h;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int wA = L.xend - L.xlim, hB = L.yend - L.ylim;
    const int64_t nA = (int64_t)wA * L.yend * p.Mz, nB = (int64_t)L.xlim * hB * p.Mz;
    int i, j, k;
    if (t < nA)
    {
        i = L.xlim + (int)(t % wA);
        j = (int)((t / wA) % L.yend);
        k = (int)(t / ((int64_t)wA * L.yend));
    }
    else if (t < nA + nB)
    {
        const int64_t u = t - nA;
        i = (int)(u % L.xlim);
        j = L.ylim + (int)((u / L.xlim) % hB);
        k = (int)(u / ((int64_t)L.xlim * hB));
    }
    else
        return;
    constexpr int B = IS_E ? 0 : 3;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        if (i < p.vlo[c][0] || i > p.vhi[c][0] || j < p.vlo[c][1] || j > p.vhi[c][1] || k < p.vlo[c][2] || k > p.vhi[c][2])
            continue;
        if (c == 0) face_point<T, B + 0>(F, i, j, k);
        else if (c == 1) face_point<T, B + 1>(F, i, j, k);
        else face_point<T, B + 2>(F, i, j, k);
    }
}
} // namespace ffipg
