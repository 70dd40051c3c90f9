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
//   TY + 1 rows).  The new H goes into a four-plane ring in shared memory,
//   on the tile and on the low-x column and low-y row that the tile's E
//   update needs (those halo points belong to neighbouring CTAs and are
//   recomputed here, not written).
//   E(k-1) needs H(k-1) and H(k-2) from that ring, written by every thread
//   in earlier iterations.  There is no block barrier in the march: every
//   thread arrives on a per-ring-plane mbarrier once its H is written, and
//   waits at the top of iteration q for all threads' H(q-1).  That one wait
//   orders the ring (with four planes, H(k) overwrites the plane that E read
//   two iterations ago) and frees the TMA stages for refill (the E stage of
//   plane q-3, the H stage of plane q-1), while a thread that finished early
//   can run ahead by an E update.
// Every field value is read from HBM once and written once per time step.
// Because neighbouring CTAs read the previous level while this CTA writes the
// new one, field buffers (and the H-side CPML psi and pole state) ping-pong
// between steps; E-side CPML psi and polarisation state are only touched by
// their owner and are updated in place.  Each chunk starts by recomputing H
// of the plane below it (no field writes).  H sources waiting at slots with
// poles are read, not cleared (the engine clears them after the pass).
//
// Two code paths per side and plane.  The common one (a tile plane with no
// CPML, no material slot, no DFT unit, every point valid) is the plain curl
// update.  The general one gates stores by per-thread validity bits (one per
// component), takes the CPML coefficients from per-axis tables staged in
// shared memory (E components use only parity-0 positions along their curl
// axes and H components only parity-1 positions, so one (b, c, 1/k) triple
// per axis and side) and handles material slots and DFT sums; its psi values
// are loaded at the top of the iteration, before the TMA wait.  A lean copy
// of it serves CPML tile planes whose points are all valid and hold no slot
// (in fp64 one copy per set of axes with CPML at the plane).  The choice is
// CTA-uniform (warp-uniform for E material slots) and comes from flags
// precomputed once per CTA.
//
// When the valid x (y) extent exceeds a whole number of tiles by one or two
// points, those last layers are left to k_face (two small launches after this
// pass: H then E), so that no CTA is spent on a nearly empty tile.
//
// PEC / PMC / periodic faces: the E layers whose curl reads an H ghost plane
// (the ghost holds the mirror / periodic image of the new H) are left to the
// E half of k_face too, which runs after the H ghost planes of the new level
// are filled; the pass reads E ghost planes of step n as loaded (filled at
// the end of the previous step), so the H update needs nothing else.  A
// PEC / PMC face at the low x / y end is not deferred: its ghost is +-1
// times the first column / row, which the tiles there compute and mirror
// into their halo.  On such grids the GH copy of the pass runs: the mirror,
// and the plain / lean E paths with the deferred points' stores masked.
//
// The per-point arithmetic is the same as the separate H/E kernels
// (stencil.cuh: pml_term, material_at, dft_point), so both passes give the
// same bits.  Every mbarrier wait is bounded; a thread whose wait gives up
// records an error word and returns (thread 0 after waiting, bounded, for its
// outstanding TMA copies), and the threads still waiting on the CTA's
// barriers give up in turn.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "engine.hpp"
#include "fused_plan.hpp"

namespace ffipg
{
// NPT adjacent x points per thread (vector loads and stores), TX = 32 NPT
// tile columns; TY tile rows, RPT adjacent rows per thread (8 warps of 32
// lanes, warp w owns rows RPT w .. RPT w + RPT - 1); SE / SH: TMA stages of
// the E / H plane rings; KCH: most z planes per CTA; MINB: CTAs per SM the
// register budget is sized for (tuning builds may override the defaults);
// STAGE_PSI: the CPML instance stages psi in shared memory by cp.async,
// ahead of use (fp32 only: the fp64 pass is bound by fp64 arithmetic, and
// there the copy instructions cost more than the latency they hide).  Tiles
// start at x0 = kXFirst + 32 u (u a unit of the job lists; kXFirst, the first
// index that holds grid points, is 2); the TMA box starts XOFF = 2 elements
// to the left, at a 16-byte boundary (32 u), and spans BX >= XOFF + TX + 1
// elements (x0 - XOFF .. x0 + TX), rounded up to 16 bytes; a thread's own
// points sit XOFF + NPT lane + p into a box row (8-byte aligned pairs in
// fp32).  The H ring planes hold rows of RW elements (XOFF + TX rounded up to
// 16 bytes): the low-x halo column at XOFF - 1, the tile's own points from
// XOFF on.
#ifndef FFIP_FUSED_F32_NPT
#define FFIP_FUSED_F32_NPT 2
#endif
#ifndef FFIP_FUSED_F32_NPT_PML
#define FFIP_FUSED_F32_NPT_PML 1
#endif
#ifndef FFIP_FUSED_F32_RPT
#define FFIP_FUSED_F32_RPT 1
#endif
#ifndef FFIP_FUSED_F32_SE
#define FFIP_FUSED_F32_SE 6
#endif
#ifndef FFIP_FUSED_F32_SE_X2
#define FFIP_FUSED_F32_SE_X2 5
#endif
#ifndef FFIP_FUSED_F32_SH
#define FFIP_FUSED_F32_SH 3
#endif
#ifndef FFIP_FUSED_F32_MINB
#define FFIP_FUSED_F32_MINB 3
#endif
#ifndef FFIP_FUSED_F32_MINB_X2
#define FFIP_FUSED_F32_MINB_X2 2
#endif
#ifndef FFIP_FUSED_F32_STAGE_PSI
#define FFIP_FUSED_F32_STAGE_PSI 1
#endif
// with STAGE_PSI: the H-side psi of the own points is staged too, copied by
// cp.async right after the H update of the iteration before the one that
// uses it (a tuning switch)
#ifndef FFIP_FUSED_F32_STAGE_PSIH
#define FFIP_FUSED_F32_STAGE_PSIH 0
#endif
#ifndef FFIP_FUSED_F64_RPT
#define FFIP_FUSED_F64_RPT 1
#endif
#ifndef FFIP_FUSED_F64_SE
#define FFIP_FUSED_F64_SE 5
#endif
#ifndef FFIP_FUSED_F64_SH
#define FFIP_FUSED_F64_SH 3
#endif
#ifndef FFIP_FUSED_F64_MINB
#define FFIP_FUSED_F64_MINB 2
#endif
// most z planes per CTA (KCH), and the shorter chunk the fp32 pass takes on
// grids that give fewer than 20 waves of CTAs at KCH planes (KCH_SHORT):
// there the shorter jobs balance the geometry-heavy ones better, on large
// grids the longer ones carry less per-job overhead; the fp64 pass (bound by
// the fp64 pipe) keeps the longer chunks
#ifndef FFIP_FUSED_KCH
#define FFIP_FUSED_KCH 16
#endif
#ifndef FFIP_FUSED_F32_KCH_SHORT
#define FFIP_FUSED_F32_KCH_SHORT 12
#endif
constexpr int fused_box_width(int xoff, int tx, int elems16) { return (xoff + tx + 1 + elems16 - 1) / elems16 * elems16; }
// The two instances (P = true: the CPML jobs, P = false: the interior jobs)
// may take different tile widths: interior jobs are TX-wide tiles of the
// interior instance's NPT; a column of that width that touches a CPML point
// runs as TX / TX_P narrower jobs of the CPML instance.
template <typename T, bool P>
struct FusedShape;
#ifndef FFIP_FUSED_F32_XOFF
#define FFIP_FUSED_F32_XOFF 2
#endif
template <bool P>
struct FusedShape<float, P>
{
    static constexpr int NPT = P ? FFIP_FUSED_F32_NPT_PML : FFIP_FUSED_F32_NPT, TX = 32 * NPT, RPT = FFIP_FUSED_F32_RPT,
                         TY = 8 * RPT, XOFF = FFIP_FUSED_F32_XOFF, BX = fused_box_width(XOFF, TX, 4),
                         RW = (XOFF + TX + 3) / 4 * 4,
                         SE = NPT == 1 ? FFIP_FUSED_F32_SE : FFIP_FUSED_F32_SE_X2, SH = FFIP_FUSED_F32_SH, KCH = FFIP_FUSED_KCH,
                         KCH_SHORT = FFIP_FUSED_F32_KCH_SHORT, MINB = NPT == 1 ? FFIP_FUSED_F32_MINB : FFIP_FUSED_F32_MINB_X2,
                         STAGE_PSI = FFIP_FUSED_F32_STAGE_PSI, STAGE_PSIH = STAGE_PSI && FFIP_FUSED_F32_STAGE_PSIH;
};
template <bool P>
struct FusedShape<double, P>
{
    static constexpr int NPT = 1, TX = 32, RPT = FFIP_FUSED_F64_RPT, TY = 8 * RPT, XOFF = 2, BX = fused_box_width(XOFF, TX, 2),
                         RW = XOFF + TX, SE = FFIP_FUSED_F64_SE, SH = FFIP_FUSED_F64_SH, KCH = FFIP_FUSED_KCH,
                         KCH_SHORT = FFIP_FUSED_KCH, MINB = FFIP_FUSED_F64_MINB, STAGE_PSI = 0, STAGE_PSIH = 0;
};

// NPT consecutive values of one row: an aligned vector load / store (float2
// for two fp32 values), elementwise otherwise
template <typename T, int N>
struct Vals
{
    T v[N];
    __device__ __forceinline__ T &operator[](int i) { return v[i]; }
    __device__ __forceinline__ const T &operator[](int i) const { return v[i]; }
};
template <int N, typename T>
__device__ __forceinline__ Vals<T, N> ldv(const T *p)
{
    Vals<T, N> r;
    if constexpr (N == 2 && sizeof(T) == 4)
    {
        const float2 f = *reinterpret_cast<const float2 *>(p);
        r.v[0] = f.x;
        r.v[1] = f.y;
    }
    else
    {
#pragma unroll
        for (int i = 0; i < N; ++i) r.v[i] = p[i];
    }
    return r;
}

template <typename T, int N>
__device__ __forceinline__ void stv(T *p, const Vals<T, N> &v)
{
    if constexpr (N == 2 && sizeof(T) == 4)
        *reinterpret_cast<float2 *>(p) = make_float2(v.v[0], v.v[1]);
    else
    {
#pragma unroll
        for (int i = 0; i < N; ++i) p[i] = v.v[i];
    }
}

// CPML instance: a warp covers 16 columns of two tile rows (see k_fused);
// 1: in both precisions; 2 (default): in fp64 only
#ifndef FFIP_FUSED_PML_SPLITWARP
#define FFIP_FUSED_PML_SPLITWARP 2
#endif
// with split warps: on a CPML tile plane whose points are all valid and hold
// no slot and no DFT unit (the lean paths), a warp whose own columns and
// rows have no CPML, on a plane without z CPML, takes the plain path (in an
// x-slab tile half the warps lie outside the slab)
#ifndef FFIP_FUSED_PML_WARP_FAST
#define FFIP_FUSED_PML_WARP_FAST 1
#endif
// PEC / PMC faces at the low x / y end mirrored into the halo of the first
// tiles (FusedLaunch::hmirror); 0: their E layers deferred like the others'
#ifndef FFIP_FUSED_HALO_MIRROR
#define FFIP_FUSED_HALO_MIRROR 1
#endif

// plain paths: x +- 1 neighbours from the adjacent lane by warp shuffle
// instead of shared memory, per instance: bit 0 the fp32 interior instance,
// bit 1 the fp32 CPML instance, bit 2 the fp64 interior instance, bit 3 the
// fp64 CPML instance (both fp32 instances together: 5 % slower on the 256^3
// workload, the shuffles' registers make them spill)
#ifndef FFIP_FUSED_SHFL
#define FFIP_FUSED_SHFL 0
#endif

// fp32 interior instance: E rows with material slots on a tile plane that
// is otherwise plain take the plain path with the slot points patched
#ifndef FFIP_FUSED_SLOT_PATCH
#define FFIP_FUSED_SLOT_PATCH 1
#endif

// the general E path of the interior instance (fp32) adds the DFT sums of
// a tile row's points together, with their loads batched
#ifndef FFIP_FUSED_DFT_DEFER
#define FFIP_FUSED_DFT_DEFER 1
#endif

// the lean CPML path is compiled per axis for tile planes with CPML along
// one axis only (fp64: bound by the fp64 pipe, every instruction left out
// counts; fp32 keeps one generic copy)
#ifndef FFIP_FUSED_F32_AXIS_SPEC
#define FFIP_FUSED_F32_AXIS_SPEC 0
#endif
template <typename T>
constexpr bool kAxisSpec = sizeof(T) == 8 || FFIP_FUSED_F32_AXIS_SPEC;
// fp64 copies for the tile planes with CPML along two axes (slab edges) as
// well as one
#ifndef FFIP_FUSED_F64_AXIS_PAIRS
#define FFIP_FUSED_F64_AXIS_PAIRS 1
#endif

// CPML coefficients of one position along one axis: b, c, 1/k, and in the
// fourth slot the bit pattern of an integer flag word, bit 0 = (c != 0) and
// (with the per-axis copies) bit 1 = (c != 0 or 1/k != 1): the CPML paths
// test these on the integer pipe (a floating-point compare issues on the
// fp64 pipe, which bounds the fp64 pass).  none(): a position without CPML
// (c = 0, 1/k = 1).
template <typename T>
struct alignas(4 * sizeof(T)) PmlCoef
{
    T b, c, ik, flagbits;
    __device__ __forceinline__ unsigned flags() const
    {
        if constexpr (sizeof(T) == 8) return (unsigned)__double2loint(flagbits);
        else return __float_as_uint(flagbits);
    }
    __device__ __forceinline__ bool nz() const
    {
        if constexpr (kAxisSpec<T>) return flags() & 1u;
        else return flags() != 0u;  // bit 0 only
    }
    __device__ __forceinline__ bool active() const
    {
        static_assert(kAxisSpec<T>, "without the per-axis copies the flag word holds bit 0 only");
        return flags() & 2u;
    }
    __device__ __forceinline__ void set_flags()
    {
        const unsigned f = kAxisSpec<T> ? (c != T(0) ? 3u : 0u) | (ik != T(1) ? 2u : 0u) : (c != T(0) ? 1u : 0u);
        if constexpr (sizeof(T) == 8) flagbits = __hiloint2double(0, (int)f);
        else flagbits = __uint_as_float(f);
    }
    __device__ __forceinline__ static PmlCoef none()
    {
        PmlCoef e;
        e.b = e.c = e.flagbits = T(0);
        e.ik = T(1);
        return e;
    }
};

template <typename T, bool P>
struct FusedLayout
{
    using SH = FusedShape<T, P>;
    static constexpr int E_BYTES = (SH::TY + 2) * SH::BX * (int)sizeof(T);  // one E box
    static constexpr int H_BYTES = (SH::TY + 1) * SH::BX * (int)sizeof(T);  // one H box
    static constexpr int E_TILE = (E_BYTES + 127) / 128 * 128;
    static constexpr int H_TILE = (H_BYTES + 127) / 128 * 128;
    static constexpr int E_OFF = 128;  // [0, 128): mbarriers
    static constexpr int H_OFF = E_OFF + SH::SE * 3 * E_TILE;
    static constexpr int HN_OFF = H_OFF + SH::SH * 3 * H_TILE;
    static constexpr int HN_PLANE = 3 * (SH::TY + 1) * SH::RW;  // elements of one H ring plane
    static constexpr int NX = SH::TX + 1, NY = SH::TY + 1, NZ = SH::KCH + 2;  // CPML table lengths
    static constexpr int PML_OFF = (HN_OFF + 4 * HN_PLANE * (int)sizeof(T) + 31) / 32 * 32;
    static constexpr int PML_BYTES = 2 * (NX + NY + NZ) * (int)sizeof(PmlCoef<T>);  // [axis][parity][n]
    static constexpr int INFO_OFF = PML_OFF + PML_BYTES;
    // CPML instance with STAGE_PSI: E-side psi of the own points staged by
    // cp.async, one slot of 256 elements (one per thread) per
    // [row][point][component][axis]
    static constexpr int PSI_OFF = (INFO_OFF + (NZ + 1) * 4 + 15) / 16 * 16;  // NZ plane words + the tile's axis word
    static constexpr int PSI_E = 0, PSI_H = 6 * SH::RPT * SH::NPT;  // E slots, then (STAGE_PSIH) H slots
    static constexpr int PSI_SLOTS = (SH::STAGE_PSI ? 6 * SH::RPT * SH::NPT : 0) + (SH::STAGE_PSIH ? 6 * SH::RPT * SH::NPT : 0);
    static constexpr int SMEM = PSI_OFF;  // the instance without CPML code
    static constexpr int SMEM_PML = PSI_OFF + PSI_SLOTS * 256 * (int)sizeof(T);
    static_assert((SH::SE + SH::SH + 5) * 8 <= 120, "mbarriers do not fit");
    static_assert(SH::SE >= 5, "E planes q-2 .. q+1 are in use while one more loads");
    static_assert(SH::BX >= SH::XOFF + SH::TX + 1, "TMA box too narrow");
    static_assert((kXFirst - SH::XOFF) * (int)sizeof(T) % 16 == 0 && SH::TX * (int)sizeof(T) % 16 == 0,
                  "TMA box start (x0 - XOFF = kXFirst - XOFF + TX bx) off a 16-byte boundary");
    static_assert(SH::BX * (int)sizeof(T) % 16 == 0, "TMA box width not a multiple of 16 bytes");
    static_assert(SH::XOFF * (int)sizeof(T) % (SH::NPT * (int)sizeof(T)) == 0 && SH::RW * (int)sizeof(T) % 16 == 0,
                  "own points of a box row / ring row not aligned for NPT-wide vector access");
    static_assert(SH::TX == 32 * SH::NPT && SH::TY == 8 * SH::RPT && 2 * SH::TY <= 32, "8 warps of 32 lanes, halo in one warp");
};

// per-plane flag word (one per plane of the chunk, shared memory); bits
// 0..TY-1: tile row r holds E material slots
constexpr unsigned kInfoZValidShift = 16;  // bits 16..21: component c valid at this z
constexpr unsigned kInfoZPml = 1u << 22;   // CPML at this tile plane: along z (either parity), or the tile's x / y
constexpr unsigned kInfoDftE = 1u << 23;   // an E DFT unit meets this tile plane
constexpr unsigned kInfoDftH = 1u << 24;   // an H DFT unit meets this tile plane
constexpr unsigned kInfoFastH = 1u << 25;  // H of this tile plane takes the plain path
constexpr unsigned kInfoFastE = 1u << 26;  // E of this tile plane takes the plain path (rows without slots)
constexpr unsigned kInfoLeanH = 1u << 27;  // H: CPML, but every point valid, no slot, no DFT unit
constexpr unsigned kInfoLeanE = 1u << 28;  // E: CPML, but every point valid, no DFT unit (rows without slots)
constexpr unsigned kInfoZeroCol = 1u << 29;  // the low-x halo column holds no grid point (the same in every plane word)
constexpr unsigned kInfoZeroRow = 1u << 30;  // the low-y halo row holds no grid point (the same in every plane word)

template <typename T>
struct FusedLaunch
{
    CUtensorMap tm_e[3];  // E input arrays, box (BX, TY + 2, 1)
    CUtensorMap tm_h[3];  // H input arrays, box (BX, TY + 1, 1)
    FusedParams<T> fp;
    int *err;             // set to 1 when a wait times out
    int xlim, ylim;       // this pass updates 1 <= x < xlim, 1 <= y < ylim; k_face the rest
    int xend, yend;       // valid extents (max over components of vhi + 1)
    int kbeg, kend;       // valid z range
    // E points of component c this pass owns along axis a: elo[c][a] ..
    // ehi[c][a], the valid range less the layers whose curl reads a ghost H
    // (PEC / PMC / periodic faces): k_face updates those after the H ghost
    // planes are refreshed
    int elo[3][3], ehi[3][3];
    // PEC / PMC face at the low x (a = 0) / y (a = 1) end: its H ghost
    // column / row hghost[a] holds hmirror[a] (+1 / -1) times the new H of the
    // first column / row, which the tiles there put into their halo (so the
    // E layer next to it stays in the pass); hmirror[a] = 0: no such face
    int hmirror[2], hghost[2];
    const int4 *jobs;     // per CTA: x0, y0, k0, k1 (tile origin and owned z planes)
};

// Bound of the waits that drain a CTA's outstanding TMA copies before it
// leaves after an error (ns); the march waits take FusedParams::wait_ns.
constexpr uint64_t kFusedDrainWaitNs = 2000000000ull;
// Suspend-time hint of one mbarrier poll (ns): a waiting thread sleeps until
// the phase completes or this time passes, instead of re-polling at once
#ifndef FFIP_FUSED_WAIT_HINT_NS
#define FFIP_FUSED_WAIT_HINT_NS 0
#endif
// Field and psi stores of the fused pass with the streaming (evict-first)
// cache hint, so that the step's output does not push the halo rows that
// neighbouring tiles still read out of L2
#ifndef FFIP_FUSED_STORE_CS
#define FFIP_FUSED_STORE_CS 0
#endif

template <typename T>
__device__ __forceinline__ void st_out(T *p, T v)
{
    if constexpr (FFIP_FUSED_STORE_CS) __stcs(p, v);
    else *p = v;
}
template <typename T, int N>
__device__ __forceinline__ void st_outv(T *p, const Vals<T, N> &v)
{
    if constexpr (N == 2 && sizeof(T) == 4)
    {
        const float2 f = make_float2(v.v[0], v.v[1]);
        if constexpr (FFIP_FUSED_STORE_CS) __stcs(reinterpret_cast<float2 *>(p), f);
        else *reinterpret_cast<float2 *>(p) = f;
    }
    else
    {
#pragma unroll
        for (int i = 0; i < N; ++i) st_out(p + i, v.v[i]);
    }
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    if constexpr (FFIP_FUSED_WAIT_HINT_NS > 0)
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity), "r"((uint32_t)FFIP_FUSED_WAIT_HINT_NS)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase of `parity` to complete; gives up (returns false) once
// limit_ns have passed on the global timer since the first poll failed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;)
    {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// one element global -> shared, asynchronous (completion per thread:
// cp_async_wait_all)
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst, const T *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)), "l"(src), "n"((int)sizeof(T)) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// Loads of the pass's small per-launch metadata (CTA jobs, CPML tables, slot
// row ranges) with an L2 evict-last policy, so that the field streaming of one
// step does not push them out of L2 before the next step reads them again
__device__ __forceinline__ uint64_t l2_keep_policy()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ int4 ld_keep(const int4 *a, uint64_t pol)
{
    int4 v;
    asm volatile("ld.global.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ int2 ld_keep(const int2 *a, uint64_t pol)
{
    int2 v;
    asm volatile("ld.global.L2::cache_hint.v2.s32 {%0, %1}, [%2], %3;" : "=r"(v.x), "=r"(v.y) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ float ld_keep(const float *a, uint64_t pol)
{
    float v;
    asm volatile("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ double ld_keep(const double *a, uint64_t pol)
{
    double v;
    asm volatile("ld.global.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
    return v;
}

// barrier 1 over warps 1..7 (224 threads) of the CTA, plain and with an OR
// reduction; warp 0 meanwhile issues the first TMA copies
__device__ __forceinline__ void bar_warps_1_7() { asm volatile("bar.sync 1, 224;" ::: "memory"); }
__device__ __forceinline__ bool bar_warps_1_7_or(bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, 224, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// all but the most recent group complete
__device__ __forceinline__ void cp_async_wait_but_last() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Per-CTA context of the fused pass
template <typename T, bool P>
struct FusedCtx
{
    using SH = FusedShape<T, P>;
    using LY = FusedLayout<T, P>;
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
    // new H, ring plane r (0..3), rows y0-1 .. y0+TY-1; column XOFF - 1 is
    // x0 - 1, column XOFF + j is x0 + j
    __device__ __forceinline__ T *hn_plane(int r, int c) const
    {
        return reinterpret_cast<T *>(smem + LY::HN_OFF) + r * LY::HN_PLANE + c * (SH::TY + 1) * SH::RW;
    }
    __device__ __forceinline__ T &hn_at(int r, int c, int row, int col) const { return hn_plane(r, c)[row * SH::RW + col]; }
    // CPML table of axis a, parity q: entry o is position first_a + o, with
    // first = x0 - 1, y0 - 1, k0 - 1
    __device__ __forceinline__ PmlCoef<T> *tab(int a, int q) const
    {
        PmlCoef<T> *base = reinterpret_cast<PmlCoef<T> *>(smem + LY::PML_OFF);
        return a == 0 ? base + q * LY::NX : a == 1 ? base + 2 * LY::NX + q * LY::NY : base + 2 * (LY::NX + LY::NY) + q * LY::NZ;
    }
    template <int A>
    __device__ __forceinline__ const PmlCoef<T> &pml_at(int q, int pos) const
    {
        const int o = A == 0 ? pos - (x0 - 1) : A == 1 ? pos - (y0 - 1) : pos - (k0 - 1);
        return tab(A, q)[o];
    }
};

// accdb increment at one point of component GC from its two curls, CPML
// coefficients taken from the staged tables (halo points)
template <typename T, bool P, int GC>
__device__ __forceinline__ T fused_term(const FusedCtx<T, P> &X, bool pml_plane, int x, int y, int k, int64_t idx, T curl1,
                                        T curl2, const T *pin1, const T *pin2, T *pout1, T *pout2)
{
    using C = CompT<GC>;
    if (!pml_plane) return curl1 - curl2;
    const PmlCoef<T> A1 = X.template pml_at<C::a1>(C::q1, pick<C::a1>(x, y, k));
    const PmlCoef<T> A2 = X.template pml_at<C::a2>(C::q2, pick<C::a2>(x, y, k));
    const bool n1 = A1.nz(), n2 = A2.nz();
    if (!n1 && !n2) return curl1 - curl2;
    return pml_combine_nz(n1, n2, A1.c, A2.c, A1.b, A2.b, A1.ik, A2.ik, curl1, curl2, pin1, pin2, pout1, pout2, idx);
}

// (a - b) / dx - (c - d) / dx of the plain curl update, 1/dx given; UNIT:
// 1/dx is 1 and the two multiplications are left out (the same bits: x * 1
// is x)
template <bool UNIT, typename T>
__device__ __forceinline__ T curl_diff(T a, T b, T c, T d, T inv)
{
    if (UNIT) return (a - b) - (c - d);
    return (a - b) * inv - (c - d) * inv;
}

// curl term of one component from its two curls with the CPML coefficients
// of its two curl axes (cv == 0 on both: plain curl, as Curl_Stepping)
template <typename T>
__device__ __forceinline__ T plane_term(const PmlCoef<T> &A1, const PmlCoef<T> &A2, bool n1, bool n2, T curl1, T curl2, T psi1,
                                        T psi2, T *ps1, T *ps2)
{
    if (!n1 && !n2) return curl1 - curl2;
    return pml_term_nz(n1, n2, A1.c, A2.c, A1.b, A2.b, A1.ik, A2.ik, curl1, curl2, psi1, psi2, ps1, ps2);
}

// H at the new level of a halo point (not owned: nothing is written),
// component GC (3..5), point (x, y) of plane k; E stages eA/eB hold planes
// k/k+1, H stage hA plane k.  Returns 0 where the component has no grid point.
template <typename T, bool P, int GC, bool UNIT = false>
__device__ __forceinline__ T fused_h_point(const FusedCtx<T, P> &X, int x, int y, int k, int eA, int eB, int hA, bool pml_plane,
                                           bool slots)
{
    using SH = FusedShape<T, P>;
    constexpr int BX = SH::BX, XOFF = SH::XOFF, c = GC - 3;
    const FusedParams<T> &F = X.L->fp;
    const SideParams<T> &PH = F.h;
    if (x < PH.vlo[c][0] || x > PH.vhi[c][0] || y < PH.vlo[c][1] || y > PH.vhi[c][1] || k < PH.vlo[c][2] ||
        k > PH.vhi[c][2])
        return T(0);
    const int o = (y - (X.y0 - 1)) * BX + x - (X.x0 - XOFF);
    T curl1, curl2;
    // UNIT: 1/dx is 1 and the multiplications are left out (the same bits)
    auto scale = [&](T d) { return UNIT ? d : d * PH.inv_dx; };
    if (c == 0)  // Hx: -(dEz/dy) + dEy/dz
    {
        const T *Ez = X.e_tile(eA, 2), *Ey = X.e_tile(eA, 1);
        curl1 = scale(Ez[o] - Ez[o + BX]);
        curl2 = scale(Ey[o] - X.e_tile(eB, 1)[o]);
    }
    else if (c == 1)  // Hy: -(dEx/dz) + dEz/dx
    {
        const T *Ex = X.e_tile(eA, 0), *Ez = X.e_tile(eA, 2);
        curl1 = scale(Ex[o] - X.e_tile(eB, 0)[o]);
        curl2 = scale(Ez[o] - Ez[o + 1]);
    }
    else  // Hz: -(dEy/dx) + dEx/dy
    {
        const T *Ey = X.e_tile(eA, 1), *Ex = X.e_tile(eA, 0);
        curl1 = scale(Ey[o] - Ey[o + 1]);
        curl2 = scale(Ex[o] - Ex[o + BX]);
    }
    const int idx = x + y * (int)PH.sy + k * (int)PH.sz;
    const T term = fused_term<T, P, GC>(X, pml_plane, x, y, k, idx, curl1, curl2, F.psih_in[c][0], F.psih_in[c][1], nullptr,
                                     nullptr);
    const T old = X.h_tile(hA, c)[o];
    T vd;
    if (!slots) return old + PH.coef_def * term;
    // not owned: the value only (the owner updates the slot's pole state)
    return material_at<T, false>(PH, PH.slot[c], slot_of(PH.slot[c], PH.My, x, y, k, idx), old, term, &vd);
}

// fused_h_point, or on the H ghost column / row of a PEC / PMC low x / y
// face the mirrored value of the first column / row (the value the ghost
// planes receive after the step)
template <typename T, bool P, int GC, bool UNIT = false, bool MIR = false>
__device__ __forceinline__ T fused_h_halo(const FusedCtx<T, P> &X, int x, int y, int k, int eA, int eB, int hA, bool pml_plane,
                                          bool slots)
{
    if constexpr (!MIR) return fused_h_point<T, P, GC, UNIT>(X, x, y, k, eA, eB, hA, pml_plane, slots);
    else
    {
    // one evaluation at the mirrored point, scaled by +-1 (exact)
    const FusedLaunch<T> &L = *X.L;
    int xe = x, ye = y, sc = 1;
    if (L.hmirror[0] && x == L.hghost[0] && x == X.x0 - 1)
    {
        xe = x + 1;
        sc = L.hmirror[0];
    }
    else if (L.hmirror[1] && y == L.hghost[1] && y == X.y0 - 1)
    {
        ye = y + 1;
        sc = L.hmirror[1];
    }
    const T v = fused_h_point<T, P, GC, UNIT>(X, xe, ye, k, eA, eB, hA, pml_plane, slots);
    return sc == 1 ? v : -v;
    }
}

// Halo H point p (0 .. NPT-1) of this thread, if any: Hz / Hx of the low-y
// row (warps 7 / 6, NPT points per lane), Hz / Hy of the low-x column (warp
// 5, lanes < TY / < 2 TY, p = 0 only), with its place (row, col) in an H
// ring plane
template <typename T, bool P>
__device__ __forceinline__ bool halo_point(const FusedCtx<T, P> &X, int wid, int lane, int p, int &hx, int &hy, int &comp,
                                           int &row, int &col)
{
    using SH = FusedShape<T, P>;
    constexpr int TY = SH::TY, NPT = SH::NPT, XOFF = SH::XOFF;
    const int j = lane * NPT + p;
    if (wid == 7) { hx = X.x0 + j; hy = X.y0 - 1; comp = 2; row = 0; col = XOFF + j; }
    else if (wid == 6) { hx = X.x0 + j; hy = X.y0 - 1; comp = 0; row = 0; col = XOFF + j; }
    else if (p == 0 && wid == 5 && lane < TY) { hx = X.x0 - 1; hy = X.y0 + lane; comp = 2; row = lane + 1; col = XOFF - 1; }
    else if (p == 0 && wid == 5 && lane < 2 * TY) { hx = X.x0 - 1; hy = X.y0 + lane - TY; comp = 1; row = lane - TY + 1; col = XOFF - 1; }
    else return false;
    return true;
}

// General H(k) at this thread's own point x0 + xi of tile row `row`:
// validity bits, CPML from the staged tables (psi values ph loaded by the
// caller), material slots, DFT.  AX: the axes (bit a) along which the tile
// plane may have CPML at its own points; the others are known to have none
// (c = 0, 1/k = 1) and their terms are left out of the code (the same bits).
template <typename T, bool P, bool FULL = true, bool UNIT = false, int AX = 7>
__device__ __forceinline__ void h_own_general(const FusedCtx<T, P> &X, int q, int row, int xi, int eA, int eB, int hA,
                                              int slot_new, unsigned vb, bool owned, bool pml, bool slots, bool dft, int idx,
                                              const T (&ph)[3][2])
{
    // FULL = false: the lean instance for CPML tile planes whose points are
    // all valid, with no material slot and no DFT unit
    if (!FULL)
    {
        vb = 63u;
        slots = dft = false;
    }
    using SH = FusedShape<T, P>;
    constexpr int BX = SH::BX;
    const FusedParams<T> &F = X.L->fp;
    const SideParams<T> &PH = F.h;
    const int offE = (row + 1) * BX + xi + SH::XOFF;
    const T idh = PH.inv_dx;
    const T *eA0 = X.e_tile(eA, 0), *eA1 = X.e_tile(eA, 1), *eA2 = X.e_tile(eA, 2);
    const T *eB0 = X.e_tile(eB, 0), *eB1 = X.e_tile(eB, 1);
    const T exa = eA0[offE], exy = eA0[offE + BX], exb = eB0[offE];
    const T eya = eA1[offE], eyx = eA1[offE + 1], eyb = eB1[offE];
    const T eza = eA2[offE], ezy = eA2[offE + BX], ezx = eA2[offE + 1];
    T curl1[3], curl2[3];
    // UNIT: 1/dx is 1 and the multiplications are left out (the same bits)
    const T m = UNIT ? T(1) : idh;
    curl1[0] = UNIT ? eza - ezy : (eza - ezy) * m;  // Hx: -(dEz/dy) + dEy/dz
    curl2[0] = UNIT ? eya - eyb : (eya - eyb) * m;
    curl1[1] = UNIT ? exa - exb : (exa - exb) * m;  // Hy: -(dEx/dz) + dEz/dx
    curl2[1] = UNIT ? eza - ezx : (eza - ezx) * m;
    curl1[2] = UNIT ? eya - eyx : (eya - eyx) * m;  // Hz: -(dEy/dx) + dEx/dy
    curl2[2] = UNIT ? exa - exy : (exa - exy) * m;
    PmlCoef<T> hc[3] = {};  // per axis, parity 1
    if (pml)
    {
        hc[0] = (AX & 1) ? X.tab(0, 1)[xi + 1] : PmlCoef<T>::none();
        hc[1] = (AX & 2) ? X.tab(1, 1)[row + 1] : PmlCoef<T>::none();
        hc[2] = (AX & 4) ? X.tab(2, 1)[q] : PmlCoef<T>::none();
    }
    auto hn = [&](int a) { return ((AX >> a) & 1) && hc[a].nz(); };
    const int x = X.x0 + xi, y = X.y0 + row, k = X.k0 - 1 + q;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        T ps1 = T(0), ps2 = T(0);
        const T term = plane_term(hc[a1], hc[a2], hn(a1), hn(a2), curl1[c], curl2[c], ph[c][0], ph[c][1], &ps1, &ps2);
        const T old = X.h_tile(hA, c)[offE];
        T v, vd;
        if (!slots)
        {
            v = old + PH.coef_def * term;
            vd = PH.g_def * v;
        }
        else
            // (on the recomputed plane below the chunk, owned = false, the
            // owner of that plane writes the same new pole state: both read
            // the old state and the same inputs)
            v = material_at(PH, PH.slot[c], slot_of(PH.slot[c], PH.My, x, y, k, idx), old, term, &vd);
        const bool val = (vb >> (3 + c)) & 1u;
        X.hn_at(slot_new, c, row + 1, SH::XOFF + xi) = val ? v : T(0);
        if (owned && val)
        {
            st_out(&F.hout[c][idx], v);
            if (hn(a1)) st_out(&F.psih_out[c][0][idx], ps1);
            if (hn(a2)) st_out(&F.psih_out[c][1][idx], ps2);
            if (dft) dft_point<T>(PH.nunits, PH.units, PH.phase, 3 + c, x, y, k, (double)v, (double)vd);
        }
    }
}

// General E(k) at this thread's own point of tile row `row` (E plane qe of
// the chunk), from the H ring planes rn (plane k) and rp (plane k-1); CPML
// psi is read from the global arrays, or (STAGED) taken from the values ps
// the caller read from its staging slots, and written back in place here;
// sl: material slot indices.
template <typename T, bool P, bool FULL = true, bool STAGED = false, bool UNIT = false, int AX = 7>
__device__ __forceinline__ void e_own_general(const FusedCtx<T, P> &X, int qe, int row, int xi, int eS, int rn, int rp,
                                              unsigned vb, bool pml, bool slots, bool dft, int idx, const int (&sl)[3],
                                              const T (&ps)[3][2], double (*dv)[2] = nullptr)
{
    using SH = FusedShape<T, P>;
    constexpr int BX = SH::BX, RW = SH::RW;
    if (!FULL)
    {
        vb &= 63u;  // every point valid (less the caller's masked ones)
        slots = dft = false;
    }
    const FusedParams<T> &F = X.L->fp;
    const SideParams<T> &PE = F.e;
    const int offE = (row + 1) * BX + xi + SH::XOFF;
    const int offN = (row + 1) * RW + xi + SH::XOFF;
    PmlCoef<T> ec[3] = {};  // per axis, parity 0
    T pe[3][2] = {};
    auto en = [&](int a) { return ((AX >> a) & 1) && ec[a].nz(); };
    if (pml)
    {
        ec[0] = (AX & 1) ? X.tab(0, 0)[xi + 1] : PmlCoef<T>::none();
        ec[1] = (AX & 2) ? X.tab(1, 0)[row + 1] : PmlCoef<T>::none();
        ec[2] = (AX & 4) ? X.tab(2, 0)[qe] : PmlCoef<T>::none();
#pragma unroll
        for (int c = 0; c < 3; ++c)
        {
            const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
            const bool ve = (vb >> c) & 1u;
            if (STAGED)
            {
                pe[c][0] = ps[c][0];
                pe[c][1] = ps[c][1];
            }
            else
            {
                if (ve && en(a1)) pe[c][0] = PE.psi[c][0][idx];
                if (ve && en(a2)) pe[c][1] = PE.psi[c][1][idx];
            }
        }
    }
    const T ide = PE.inv_dx;
    const T *n0 = X.hn_plane(rn, 0), *n1 = X.hn_plane(rn, 1), *n2 = X.hn_plane(rn, 2);
    const T *p0 = X.hn_plane(rp, 0), *p1 = X.hn_plane(rp, 1);
    const T hzr = n2[offN], hzy = n2[offN - RW], hzx = n2[offN - 1];
    const T hyr = n1[offN], hyp = p1[offN], hyx = n1[offN - 1];
    const T hxr = n0[offN], hxp = p0[offN], hxy = n0[offN - RW];
    T curl1[3], curl2[3];
    const T m = UNIT ? T(1) : ide;
    curl1[0] = UNIT ? hzr - hzy : (hzr - hzy) * m;  // Ex: dHz/dy - dHy/dz
    curl2[0] = UNIT ? hyr - hyp : (hyr - hyp) * m;
    curl1[1] = UNIT ? hxr - hxp : (hxr - hxp) * m;  // Ey: dHx/dz - dHz/dx
    curl2[1] = UNIT ? hzr - hzx : (hzr - hzx) * m;
    curl1[2] = UNIT ? hyr - hyx : (hyr - hyx) * m;  // Ez: dHy/dx - dHx/dy
    curl2[2] = UNIT ? hxr - hxy : (hxr - hxy) * m;
    const int x = X.x0 + xi, y = X.y0 + row, k = X.k0 - 1 + qe;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        T ps1 = T(0), ps2 = T(0);
        const T term = plane_term(ec[a1], ec[a2], en(a1), en(a2), curl1[c], curl2[c], pe[c][0], pe[c][1], &ps1, &ps2);
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
            st_out(&F.eout[c][idx], v);
            if (en(a1)) st_out(&PE.psi[c][0][idx], ps1);
            if (en(a2)) st_out(&PE.psi[c][1][idx], ps2);
            if (dft && !dv) dft_point<T>(PE.nunits, PE.units, PE.phase, c, x, y, k, (double)v, (double)vd);
        }
        // dv: the caller adds the DFT sums of the row's points together
        // (a point without component c adds zero)
        if (dv)
        {
            const bool val = (vb >> c) & 1u;
            dv[c][0] = val ? (double)v : 0.0;
            dv[c][1] = val ? (double)vd : 0.0;
        }
    }
}

// PML = false: the instance for jobs whose tiles, halos and planes hold no
// CPML point (the host sorts the jobs); it carries no CPML code.  GH: the
// copy launched on grids with PEC / PMC / periodic faces: the first tiles
// next to a PEC / PMC low x / y face mirror its H ghost into their halo, and
// tiles whose first column or row of an E component is deferred to the face
// kernel keep the plain and lean paths with those points' stores and DFT
// sums masked; without it the code of the other grids stays as small as
// before.
template <typename T, bool PML, bool GH = false>
__global__ void __launch_bounds__(256, FusedShape<T, PML>::MINB) k_fused(const __grid_constant__ FusedLaunch<T> L)
{
    using SH = FusedShape<T, PML>;
    using LY = FusedLayout<T, PML>;
    constexpr int TX = SH::TX, TY = SH::TY, RPT = SH::RPT, NPT = SH::NPT, XOFF = SH::XOFF, SE = SH::SE, SHS = SH::SH,
                  BX = SH::BX, RW = SH::RW;
    constexpr int NTH = 256;
    extern __shared__ __align__(128) unsigned char smem[];
    const FusedParams<T> &F = L.fp;
    const SideParams<T> &PE = F.e;
    const SideParams<T> &PH = F.h;
    const int lane = threadIdx.x, wid = threadIdx.y, tid = wid * 32 + lane;
    // own points of a thread: column ol (NPT points from ol NPT) of tile row
    // r0 (RPT rows).  SPLITW (the CPML instance, one point and one row per
    // thread): warp w covers 16 columns of two rows (columns 16 (w & 1) ..),
    // so that in a tile whose first half lies in the x slab the CPML work
    // falls to whole warps instead of half-masked ones; in fp64 rows
    // 2 (w >> 1) and 2 (w >> 1) + 1, in fp32 rows (w >> 1) and (w >> 1) + 4
    // (shared-memory rows of 36 words: four rows apart, the two half-warps
    // fall on disjoint banks; adjacent rows would overlap on 12 of them);
    // otherwise warp w covers row w, one column per lane
    constexpr bool SPLITW = (FFIP_FUSED_PML_SPLITWARP == 1 || (FFIP_FUSED_PML_SPLITWARP == 2 && sizeof(T) == 8)) && PML &&
                            NPT == 1 && RPT == 1 && SH::TX == 32;
    // warp-shuffle neighbours in this instance (lanes along x: not with SPLITW)
    constexpr bool SHFL = ((FFIP_FUSED_SHFL >> ((sizeof(T) == 8 ? 2 : 0) + (PML ? 1 : 0))) & 1) && !SPLITW;
    const int ol = SPLITW ? (lane & 15) + 16 * (wid & 1) : lane;
    constexpr int SPLIT_RS = sizeof(T) == 4 ? 4 : 1;  // SPLITW: rows of a warp this far apart
    static_assert(!SPLITW || sizeof(T) == 8 || (SH::RW % 32 == 4 && SH::BX % 32 == 4 && SH::TY == 8),
                  "fp32 split warps: the row pairing assumes rows of 36 words and 8-row tiles");
    const int r0 = SPLITW ? (SPLIT_RS == 1 ? 2 * (wid >> 1) : (wid >> 1)) + SPLIT_RS * (lane >> 4)
                          : wid * RPT;  // first tile row of this thread
    FusedCtx<T, PML> X;
    X.smem = smem;
    X.L = &L;
    const uint64_t keep = l2_keep_policy();
    const int4 job = ld_keep(L.jobs + blockIdx.x, keep);
    X.x0 = job.x;
    X.y0 = job.y;
    X.k0 = job.z;
    const int k1 = job.w;
    const int NP = k1 - X.k0 + 2;  // planes k0-1 .. k1 (plane p is z = k0 - 1 + p)
    uint64_t *ebar = reinterpret_cast<uint64_t *>(smem);
    uint64_t *hbar = ebar + SE;
    uint64_t *hd = hbar + SHS;  // per H ring plane: every thread has written its H there
    uint64_t *stall = hd + 4;   // completed by nothing (the timeout path under test)

    if (tid == 0)
    {
        for (int s = 0; s < SE; ++s) mbar_init(&ebar[s], 1);
        for (int s = 0; s < SHS; ++s) mbar_init(&hbar[s], 1);
        for (int s = 0; s < 4; ++s) mbar_init(&hd[s], NTH);
        mbar_init(stall, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if constexpr (kAxisSpec<T>) reinterpret_cast<unsigned *>(smem + LY::INFO_OFF)[LY::NZ] = 0u;  // the tile's axis word
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
    // E planes 0 .. NP-1 are used; H planes 0 .. NP-2.  Warp 0 issues the
    // first copies, the planes the first iterations wait for first (E0, E1,
    // H0, E2, H1, ...), while warps 1..7 stage the tables and flag words
    // below (barrier 1 among themselves); everyone meets at the end.
    int e_issued = min(SE, NP), h_issued = min(SHS, NP - 1);
    if (tid == 0)
    {
        int pe = 0, ph = 0;
        while (pe < e_issued || ph < h_issued)
        {
            if (pe < e_issued && (pe <= ph + 1 || ph >= h_issued)) issue_e(pe++);
            else issue_h(ph++);
        }
    }
    const bool pml_tables = PML && PE.pc[0][0] != nullptr;
    constexpr int PT = NTH - 32;   // threads of warps 1..7
    const int pt = tid - 32;        // this thread's index among them (< 0 in warp 0)
    unsigned *info = reinterpret_cast<unsigned *>(smem + LY::INFO_OFF);
    const bool h_slots = PH.slot[0].map || PH.slot[1].map || PH.slot[2].map;
    if (wid > 0)
    {
    // stage the CPML tables of this tile / chunk while the first planes load
    bool tile_pml = false;
    if (pml_tables)
    {
        for (int a = 0; a < 3; ++a)
        {
            const int n = a == 0 ? LY::NX : a == 1 ? LY::NY : LY::NZ;
            const int first = a == 0 ? X.x0 - 1 : a == 1 ? X.y0 - 1 : X.k0 - 1;
            const int len = a == 0 ? L.xend : a == 1 ? PE.My : PE.Mz;  // table lengths (x: valid extent, not the padded row)
            for (int t = pt; t < 2 * n; t += PT)
            {
                const int q = t / n, o = t % n, pos = first + o;
                const bool in = pos >= 0 && pos < len;
                PmlCoef<T> e;
                e.b = in ? ld_keep(PE.pb[a][q] + pos, keep) : T(0);
                e.c = in ? ld_keep(PE.pc[a][q] + pos, keep) : T(0);
                e.ik = in ? ld_keep(PE.pik[a][q] + pos, keep) : T(1);
                e.set_flags();
                X.tab(a, q)[o] = e;
                if (a < 2 && e.nz()) tile_pml = true;
                // fp64: axis word, bit 2 q + a: CPML (c != 0 or 1/k != 1) along
                // x / y at an own position of the tile
                if constexpr (kAxisSpec<T>)
                    if (a < 2 && o >= 1 && o <= (a == 0 ? TX : TY) && e.active()) atomicOr(&info[LY::NZ], 1u << (2 * q + a));
            }
        }
    }
    // per plane of the chunk: flag word (z validity, CPML at the tile plane,
    // DFT units meeting the tile plane, tile rows with E material slots)
    for (int o = pt; o < LY::NZ; o += PT)
    {
        const int k = X.k0 - 1 + o;
        unsigned w = 0;
        for (int c = 0; c < 3; ++c)
        {
            if (k >= L.elo[c][2] && k <= L.ehi[c][2]) w |= 1u << (kInfoZValidShift + c);
            if (k >= PH.vlo[c][2] && k <= PH.vhi[c][2]) w |= 1u << (kInfoZValidShift + 3 + c);
        }
        if (pml_tables && k >= 0 && k < PE.Mz && (ld_keep(PE.pc[2][0] + k, keep) != T(0) || ld_keep(PE.pc[2][1] + k, keep) != T(0)))
            w |= kInfoZPml;
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
    bar_warps_1_7();
    for (int t = pt; t < LY::NZ * TY * 3; t += PT)
    {
        const int c = t % 3, r = (t / 3) % TY, o = t / (3 * TY);
        const int kk = X.k0 - 1 + o, yy = X.y0 + r;
        if (!PE.slot[c].map || kk < 0 || kk >= PE.Mz || yy >= PE.My) continue;
        const int2 rr = ld_keep(reinterpret_cast<const int2 *>(PE.slot[c].rows + yy + (int64_t)kk * PE.My), keep);
        if (rr.x <= rr.y && rr.x < X.x0 + TX && rr.y >= X.x0) atomicOr(&info[o], 1u << r);
    }
    tile_pml = bar_warps_1_7_or(tile_pml);
    // the low-x halo column / low-y halo row holds no grid point of any
    // component (the ghost layer below the first tile): the plain path takes
    // its new H as zero, as the general path does
    bool zcol = true, zrow = true;
    for (int c = 0; c < 3; ++c)
    {
        zcol = zcol && X.x0 - 1 < PE.vlo[c][0] && X.x0 - 1 < PH.vlo[c][0];
        zrow = zrow && X.y0 - 1 < PE.vlo[c][1] && X.y0 - 1 < PH.vlo[c][1];
    }
    // every own point of the tile valid in x and y for all six components,
    // and every halo point too unless its whole column / row is the ghost layer
    bool inside = X.x0 + TX <= L.xlim && X.y0 + TY <= L.ylim;
    for (int c = 0; c < 3; ++c)
        inside = inside && PE.vlo[c][0] <= X.x0 - (zcol ? 0 : 1) && X.x0 + TX - 1 <= PE.vhi[c][0] &&
                 PE.vlo[c][1] <= X.y0 - (zrow ? 0 : 1) && X.y0 + TY - 1 <= PE.vhi[c][1] &&
                 PH.vlo[c][0] <= X.x0 - (zcol ? 0 : 1) && X.x0 + TX - 1 <= PH.vhi[c][0] &&
                 PH.vlo[c][1] <= X.y0 - (zrow ? 0 : 1) && X.y0 + TY - 1 <= PH.vhi[c][1];
    // (E points left to the face kernel, the first column / row of a
    // component next to a deferred ghost, are masked on the plain and lean
    // paths: GH; without ghost faces every valid E point is owned)
    // per plane: may each side take the plain path; kInfoZPml becomes "CPML
    // at this tile plane" (the tile's x / y tables or the plane's z)
    for (int o = pt; o < LY::NZ; o += PT)
    {
        const unsigned w = info[o];
        const bool zpml = pml_tables && (tile_pml || (w & kInfoZPml));
        // the plain paths also serve planes that a DFT unit meets (they add
        // the sums of the unit's points); the lean CPML paths do not
        const bool hok = inside && !h_slots && ((w >> (kInfoZValidShift + 3)) & 7u) == 7u;
        const bool eok = inside && ((w >> kInfoZValidShift) & 7u) == 7u;
        const bool hlean = hok && !(w & kInfoDftH), elean = eok && !(w & kInfoDftE);
        info[o] = w | (zpml ? kInfoZPml : 0u) | (hok && !zpml ? kInfoFastH : 0u) | (hlean && zpml ? kInfoLeanH : 0u) |
                  (eok && !zpml ? kInfoFastE : 0u) | (elean && zpml ? kInfoLeanE : 0u) | (zcol ? kInfoZeroCol : 0u) |
                  (zrow ? kInfoZeroRow : 0u);
    }
    }

    const int x = X.x0 + ol * NPT;  // first own point of this thread
    // per own row and point: components with a grid point at (x + p, y) that
    // this pass owns
    unsigned vxy[RPT][NPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r)
#pragma unroll
        for (int p = 0; p < NPT; ++p)
        {
            const int y = X.y0 + r0 + r, xp = x + p;
            vxy[r][p] = 0;
            if (xp < L.xlim && y < L.ylim)
                for (int c = 0; c < 3; ++c)
                {
                    if (xp >= L.elo[c][0] && xp <= L.ehi[c][0] && y >= L.elo[c][1] && y <= L.ehi[c][1]) vxy[r][p] |= 1u << c;
                    if (xp >= PH.vlo[c][0] && xp <= PH.vhi[c][0] && y >= PH.vlo[c][1] && y <= PH.vhi[c][1])
                        vxy[r][p] |= 1u << (3 + c);
                }
        }
    // GH: per own row and point, the E components whose point is valid but
    // left to the face kernel (the plain and lean paths skip its store and
    // DFT sums)
    unsigned dm[RPT][NPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r)
#pragma unroll
        for (int p = 0; p < NPT; ++p)
        {
            dm[r][p] = 0;
            if constexpr (GH)
            {
                const int y = X.y0 + r0 + r, xp = x + p;
                if (xp < L.xlim && y < L.ylim)
                    for (int c = 0; c < 3; ++c)
                        if (xp >= PE.vlo[c][0] && xp <= PE.vhi[c][0] && y >= PE.vlo[c][1] && y <= PE.vhi[c][1] && !((vxy[r][p] >> c) & 1u))
                            dm[r][p] |= 1u << c;
            }
        }
    __syncthreads();
    const int sz = (int)PE.sz, sy = (int)PE.sy;
    const int own0 = x + (X.y0 + r0) * sy;              // first own point of row r0 at z = 0
    const int offE = (r0 + 1) * BX + XOFF + ol * NPT;  // first own point of row r0 in an E or H box
    const int offN = (r0 + 1) * RW + XOFF + ol * NPT;  // first own point of row r0 in an H ring plane
    const T coefH = PH.coef_def, coefE = PE.coef_def, idh = PH.inv_dx, ide = PE.inv_dx;
    // fp64: the plain path without the 1/dx multiplications when 1/dx is 1
    // (the pass is bound by the fp64 pipe there)
    const bool unit_dx = sizeof(T) == 8 && idh == T(1) && ide == T(1);
    // split warps, CPML instance: no CPML along x at the warp's columns and
    // along y at its rows (either parity), the same for all its lanes
    constexpr bool WFAST = PML && SPLITW && FFIP_FUSED_PML_WARP_FAST;
    bool warp_plain = false;
    if constexpr (WFAST)
    {
        const bool mine = pml_tables && !X.tab(0, 0)[ol + 1].nz() && !X.tab(0, 1)[ol + 1].nz() && !X.tab(1, 0)[r0 + 1].nz() &&
                          !X.tab(1, 1)[r0 + 1].nz();
        warp_plain = __all_sync(0xffffffffu, mine);
    }
    // the rows of this thread's warp (the path choices stay warp-uniform)
    const unsigned rowmask = !SPLITW ? ((1u << RPT) - 1u) << r0
                             : SPLIT_RS == 1 ? 3u << (2 * (wid >> 1))
                                             : (1u << (wid >> 1)) | (1u << ((wid >> 1) + 4));
    // fp64: axes x / y (bits 0 / 1) with CPML at the tile's own points, per side
    const unsigned axw = kAxisSpec<T> && PML ? info[LY::NZ] : 0u;
    const int ax_e = (int)(axw & 3u), ax_h = (int)((axw >> 2) & 3u);

    // material slot indices of the E plane of the next iteration, loaded one
    // iteration ahead (rows flagged in the plane word only)
    int sl_next[RPT][NPT][3];
#pragma unroll
    for (int r = 0; r < RPT; ++r)
#pragma unroll
        for (int p = 0; p < NPT; ++p) sl_next[r][p][0] = sl_next[r][p][1] = sl_next[r][p][2] = -1;
    // running ring positions: E stages of planes q-1, q, q+1; H stage of
    // plane q; H ring planes of H(k), H(k-1), H(k-2)
    int eS = SE - 1, eA = 0, eB = 1 % SE, hA = 0, rn = 0, rp = 3, rpp = 2;
    int idx = own0 + (X.k0 - 1) * sz;
    // psi staging of the CPML instance (fp32): the E-side psi of the own
    // points of iteration q is copied by cp.async at the top of the
    // iteration, during the waits and the H update
    constexpr bool STG = PML && SH::STAGE_PSI;
    // STGH: the H-side psi of iteration q + 1 is copied after the H update of
    // iteration q (its own group, after the E group of iteration q, so that
    // "all but the last group" waits for the E psi before the E update and
    // for the H psi at the next H update)
    constexpr bool STGH = PML && SH::STAGE_PSIH;
    T *pstage = reinterpret_cast<T *>(smem + LY::PSI_OFF) + tid;
    auto stage_slot = [&](int r, int p, int c, int a) { return pstage + (LY::PSI_E + ((r * NPT + p) * 3 + c) * 2 + a) * NTH; };
    auto stage_slot_h = [&](int r, int p, int c, int a) { return pstage + (LY::PSI_H + ((r * NPT + p) * 3 + c) * 2 + a) * NTH; };
    // iteration q: H at plane k = k0 - 1 + q (q <= NP - 2), E at plane k - 1 (q >= 2)
    for (int q = 0; q < NP; ++q, idx += sz)
    {
        int sl_e[RPT][NPT][3];
#pragma unroll
        for (int r = 0; r < RPT; ++r)
#pragma unroll
            for (int p = 0; p < NPT; ++p)
                for (int c = 0; c < 3; ++c) sl_e[r][p][c] = sl_next[r][p][c];
        const bool do_h = q <= NP - 2, do_e = q >= 2;
        const int k = X.k0 - 1 + q;
        const int idx_e = idx - sz;
        const unsigned wh = info[q], we = q >= 1 ? info[q - 1] : 0u;
        const bool e_slots = (we & rowmask) != 0u;
        const bool fast_h = wh & kInfoFastH;
        // E rows with material slots on an otherwise plain tile plane: the
        // plain path with the slot points patched (fp32 interior instance)
        const bool fast_e_sl = FFIP_FUSED_SLOT_PATCH && !PML && sizeof(T) == 4 && (we & kInfoFastE) && e_slots;
        const bool fast_e = ((we & kInfoFastE) && !e_slots) || fast_e_sl;
        const bool lean_h = PML && (wh & kInfoLeanH);
        const bool lean_e = PML && (we & kInfoLeanE) && !e_slots;
        const bool pml_h = !fast_h && pml_tables && (wh & kInfoZPml);
        const bool pml_e = !fast_e && pml_tables && (we & kInfoZPml);
        const bool dft_h = wh & kInfoDftH, dft_e = we & kInfoDftE;
        // CPML psi of this iteration's own H points, loaded before the TMA wait
        T ph[RPT][NPT][3][2];
#pragma unroll
        for (int r = 0; r < RPT; ++r)
#pragma unroll
            for (int p = 0; p < NPT; ++p)
                for (int c = 0; c < 3; ++c) ph[r][p][c][0] = ph[r][p][c][1] = T(0);
        if (do_h && pml_h && !(STGH && q >= 1))
        {
            const bool cz = X.tab(2, 1)[q].nz();  // H side (parity 1): c != 0
#pragma unroll
            for (int r = 0; r < RPT; ++r)
#pragma unroll
                for (int p = 0; p < NPT; ++p)
                {
                    const bool ch[3] = {X.tab(0, 1)[ol * NPT + p + 1].nz(), X.tab(1, 1)[r0 + r + 1].nz(), cz};
                    const unsigned vb = vxy[r][p] & (wh >> kInfoZValidShift);
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                    {
                        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
                        const bool vh = (vb >> (3 + c)) & 1u;
                        if (vh && ch[a1]) ph[r][p][c][0] = F.psih_in[c][0][idx + r * sy + p];
                        if (vh && ch[a2]) ph[r][p][c][1] = F.psih_in[c][1][idx + r * sy + p];
                    }
                }
        }
#pragma unroll
        for (int r = 0; r < RPT; ++r)
#pragma unroll
            for (int p = 0; p < NPT; ++p) sl_next[r][p][0] = sl_next[r][p][1] = sl_next[r][p][2] = -1;
        // CPML psi of this iteration's own E points (plane k - 1; updated in
        // place by this thread only), copied during the waits and the H update
        if (STG && do_e && pml_e)
        {
            const bool cz = X.tab(2, 0)[q - 1].nz();  // E side (parity 0): c != 0
#pragma unroll
            for (int r = 0; r < RPT; ++r)
#pragma unroll
                for (int p = 0; p < NPT; ++p)
                {
                    const bool ce[3] = {X.tab(0, 0)[ol * NPT + p + 1].nz(), X.tab(1, 0)[r0 + r + 1].nz(), cz};
                    const unsigned vb = vxy[r][p] & (we >> kInfoZValidShift);
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                    {
                        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
                        const bool ve = (vb >> c) & 1u;
                        if (ve && ce[a1]) cp_async_elem(stage_slot(r, p, c, 0), PE.psi[c][0] + idx_e + r * sy + p);
                        if (ve && ce[a2]) cp_async_elem(stage_slot(r, p, c, 1), PE.psi[c][1] + idx_e + r * sy + p);
                    }
                }
        }
        if (STG) cp_async_commit();
        if (q >= 1 && q <= NP - 2 && (wh & rowmask))
        {
#pragma unroll
            for (int r = 0; r < RPT; ++r)
#pragma unroll
                for (int p = 0; p < NPT; ++p)
                {
                    const unsigned vb = vxy[r][p] & (wh >> kInfoZValidShift);
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        if (PE.slot[c].map && ((vb >> c) & 1u)) sl_next[r][p][c] = PE.slot[c].map[idx + r * sy + p];
                }
        }
        // every thread has written H(q-1): the ring plane of H(q-2) is read
        // and the one of H(k-3) free, the E stage of plane q-3 and the H
        // stage of plane q-1 are no longer read by anyone
        bool ok = q == 0 || mbar_wait_bounded(&hd[(q - 1) & 3], ((q - 1) >> 2) & 1, F.wait_ns);
        // the timeout path under test: a barrier that nothing completes
        if (q == 0 && F.stall_test) ok = mbar_wait_bounded(stall, 0, F.wait_ns);
        if (tid == 0 && ok)
        {
            bool fence = false;
            if (q >= 3 && q - 3 + SE < NP)
            {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                fence = true;
                issue_e(q - 3 + SE);
                e_issued = q - 2 + SE;
            }
            if (q >= 1 && q - 1 + SHS <= NP - 2)
            {
                if (!fence) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_h(q - 1 + SHS);
                h_issued = q + SHS;
            }
        }
        if (ok && q == 0) ok = mbar_wait_bounded(&ebar[0], 0, F.wait_ns);
        if (ok && q + 1 < NP) ok = mbar_wait_bounded(&ebar[(q + 1) % SE], ((q + 1) / SE) & 1, F.wait_ns);
        if (ok && do_h) ok = mbar_wait_bounded(&hbar[q % SHS], (q / SHS) & 1, F.wait_ns);
        if (!ok)
        {
            // a wait gave up: record it, let thread 0 wait (bounded) for its
            // copies, and leave; threads still waiting on this CTA's
            // barriers give up in turn
            atomicExch(L.err, 1);
            cp_async_wait_all();
            if (tid == 0)
            {
                for (int p = 0; p < e_issued; ++p) mbar_wait_bounded(&ebar[p % SE], (p / SE) & 1, kFusedDrainWaitNs);
                for (int p = 0; p < h_issued; ++p) mbar_wait_bounded(&hbar[p % SHS], (p / SHS) & 1, kFusedDrainWaitNs);
            }
            return;
        }
        // STGH: this iteration's H-side psi from its staging slots (the last
        // group, this iteration's E psi, may still be in flight)
        if (STGH && do_h && pml_h && q >= 1)
        {
            cp_async_wait_but_last();
            const bool cz = X.tab(2, 1)[q].nz();
#pragma unroll
            for (int r = 0; r < RPT; ++r)
#pragma unroll
                for (int p = 0; p < NPT; ++p)
                {
                    const bool ch[3] = {X.tab(0, 1)[ol * NPT + p + 1].nz(), X.tab(1, 1)[r0 + r + 1].nz(), cz};
                    const unsigned vb = vxy[r][p] & (wh >> kInfoZValidShift);
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                    {
                        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
                        const bool vh = (vb >> (3 + c)) & 1u;
                        if (vh && ch[a1]) ph[r][p][c][0] = *stage_slot_h(r, p, c, 0);
                        if (vh && ch[a2]) ph[r][p][c][1] = *stage_slot_h(r, p, c, 1);
                    }
                }
        }
        // 1. H(k) at the tile's own points, and the halo the E update of the
        //    next iteration reads: Hz, Hx on the low-y row (warps 7, 6), Hz,
        //    Hy on the low-x column (warp 5) (recomputed, not written)
        // the lean planes' halo H (general code, also after a warp's plain
        // own points)
        auto general_halo = [&]() {
#pragma unroll
            for (int p = 0; p < NPT; ++p)
            {
                int hx, hy, comp, row, col;
                if (halo_point(X, wid, lane, p, hx, hy, comp, row, col))
                {
                    auto halo = [&](auto unit) {
                        constexpr bool U = decltype(unit)::value;
                        if (comp == 0) return fused_h_halo<T, PML, 3, U, GH>(X, hx, hy, k, eA, eB, hA, pml_h, h_slots);
                        if (comp == 1) return fused_h_halo<T, PML, 4, U, GH>(X, hx, hy, k, eA, eB, hA, pml_h, h_slots);
                        return fused_h_halo<T, PML, 5, U, GH>(X, hx, hy, k, eA, eB, hA, pml_h, h_slots);
                    };
                    T v;
                    if constexpr (sizeof(T) == 8)
                        v = unit_dx ? halo(std::true_type{}) : halo(std::false_type{});
                    else
                        v = halo(std::false_type{});
                    X.hn_at(rn, comp, row, col) = v;
                }
            }
        };
        const bool warp_fast_h = WFAST && lean_h && warp_plain && !X.tab(2, 1)[q].nz();
        if (do_h)
        {
            if (fast_h || warp_fast_h)
            {
                auto fast_h_own = [&](auto unit) {
                    constexpr bool U = decltype(unit)::value;
                    const T *eA0 = X.e_tile(eA, 0) + offE, *eA1 = X.e_tile(eA, 1) + offE, *eA2 = X.e_tile(eA, 2) + offE;
                    const T *eB0 = X.e_tile(eB, 0) + offE, *eB1 = X.e_tile(eB, 1) + offE;
                    const T *hA0 = X.h_tile(hA, 0) + offE, *hA1 = X.h_tile(hA, 1) + offE, *hA2 = X.h_tile(hA, 2) + offE;
                    Vals<T, NPT> exa[RPT + 1], eza[RPT + 1];
#pragma unroll
                    for (int r = 0; r <= RPT; ++r)
                    {
                        exa[r] = ldv<NPT>(eA0 + r * BX);
                        eza[r] = ldv<NPT>(eA2 + r * BX);
                    }
                    Vals<T, NPT> hn0[RPT], hn1[RPT], hn2[RPT];
#pragma unroll
                    for (int r = 0; r < RPT; ++r)
                    {
                        const Vals<T, NPT> eya = ldv<NPT>(eA1 + r * BX), eyb = ldv<NPT>(eB1 + r * BX), exb = ldv<NPT>(eB0 + r * BX);
                        const Vals<T, NPT> h0 = ldv<NPT>(hA0 + r * BX), h1 = ldv<NPT>(hA1 + r * BX), h2 = ldv<NPT>(hA2 + r * BX);
                        // x + 1 neighbours: the next point of the pair, or the
                        // next lane's first point (warp shuffle; the last lane
                        // reads the box column after the tile)
                        T eyn, ezn;
                        if constexpr (SHFL)
                        {
                            eyn = __shfl_down_sync(0xffffffffu, eya[0], 1);
                            ezn = __shfl_down_sync(0xffffffffu, eza[r][0], 1);
                            if (lane == 31)
                            {
                                eyn = eA1[r * BX + NPT];
                                ezn = eA2[r * BX + NPT];
                            }
                        }
                        else
                        {
                            eyn = eA1[r * BX + NPT];
                            ezn = eA2[r * BX + NPT];
                        }
#pragma unroll
                        for (int p = 0; p < NPT; ++p)
                        {
                            const T eyx = p + 1 < NPT ? eya[p + 1] : eyn, ezx = p + 1 < NPT ? eza[r][p + 1] : ezn;
                            hn0[r][p] = h0[p] + coefH * curl_diff<U>(eza[r][p], eza[r + 1][p], eya[p], eyb[p], idh);
                            hn1[r][p] = h1[p] + coefH * curl_diff<U>(exa[r][p], exb[p], eza[r][p], ezx, idh);
                            hn2[r][p] = h2[p] + coefH * curl_diff<U>(eya[p], eyx, exa[r][p], exa[r + 1][p], idh);
                        }
                    }
                    T *n0 = X.hn_plane(rn, 0) + offN, *n1 = X.hn_plane(rn, 1) + offN, *n2 = X.hn_plane(rn, 2) + offN;
#pragma unroll
                    for (int r = 0; r < RPT; ++r)
                    {
                        stv(n0 + r * RW, hn0[r]);
                        stv(n1 + r * RW, hn1[r]);
                        stv(n2 + r * RW, hn2[r]);
                    }
                    if (q >= 1)
                    {
#pragma unroll
                        for (int r = 0; r < RPT; ++r)
                        {
                            st_outv(&F.hout[0][idx + r * sy], hn0[r]);
                            st_outv(&F.hout[1][idx + r * sy], hn1[r]);
                            st_outv(&F.hout[2][idx + r * sy], hn2[r]);
                        }
                        // DFT sums of the points of the tile plane that a unit
                        // meets (D/B value: g_inf of the default medium times H)
                        if (dft_h)
                            for (int r = 0; r < RPT; ++r)
                                for (int c = 0; c < 3; ++c)
                                {
                                    const Vals<T, NPT> &hv = c == 0 ? hn0[r] : c == 1 ? hn1[r] : hn2[r];
                                    double v[NPT], vd[NPT];
#pragma unroll
                                    for (int p = 0; p < NPT; ++p)
                                    {
                                        v[p] = (double)hv[p];
                                        vd[p] = (double)(PH.g_def * hv[p]);
                                    }
                                    // (the CPML instance adds its few such sums one at a
                                    // time: no call from its loop)
                                    if constexpr (PML || NPT == 1)
                                        for (int p = 0; p < NPT; ++p)
                                            dft_point<T>(PH.nunits, PH.units, PH.phase, 3 + c, x + p, X.y0 + r0 + r, k, v[p], vd[p]);
                                    else
                                        dft_points<NPT>(PH.nunits, PH.units, PH.phase, 3 + c, x, X.y0 + r0 + r, k, v, vd);
                                }
                    }
                };
                if constexpr (sizeof(T) == 8)
                {
                    if (unit_dx) fast_h_own(std::true_type{});
                    else fast_h_own(std::false_type{});
                }
                else
                    fast_h_own(std::false_type{});
                if (WFAST && !fast_h)
                    general_halo();
                else
                {
                const T *gA0 = X.e_tile(eA, 0), *gA1 = X.e_tile(eA, 1), *gA2 = X.e_tile(eA, 2), *gB0 = X.e_tile(eB, 0),
                        *gB1 = X.e_tile(eB, 1);
                auto fast_h_halo = [&](auto unit) {
                    constexpr bool U = decltype(unit)::value;
                    // Hz / Hx / Hy at box offset o (fast-path arithmetic)
                    auto hz = [&](int o) { return X.h_tile(hA, 2)[o] + coefH * curl_diff<U>(gA1[o], gA1[o + 1], gA0[o], gA0[o + BX], idh); };
                    auto hx = [&](int o) { return X.h_tile(hA, 0)[o] + coefH * curl_diff<U>(gA2[o], gA2[o + BX], gA1[o], gB1[o], idh); };
                    auto hy = [&](int o) { return X.h_tile(hA, 1)[o] + coefH * curl_diff<U>(gA0[o], gB0[o], gA2[o], gA2[o + 1], idh); };
                    if (wid >= 6)
                    {
                        // a PEC / PMC low y face: the row holds the mirrored first
                        // row (one evaluation, at row y0, negated for -1)
                        const bool mir = GH && L.hmirror[1] && X.y0 - 1 == L.hghost[1];
                        const bool neg = mir && L.hmirror[1] < 0, zero = !mir && (wh & kInfoZeroRow);
                        const int sh = mir ? BX : 0;
#pragma unroll
                        for (int p = 0; p < NPT; ++p)
                        {
                            const int o = XOFF + lane * NPT + p + sh;  // row y0 - 1 of the boxes (y0: mirrored)
                            const T v = zero ? T(0) : wid == 7 ? hz(o) : hx(o);
                            X.hn_at(rn, wid == 7 ? 2 : 0, 0, o - sh) = neg ? -v : v;
                        }
                    }
                    else if (wid == 5 && lane < 2 * TY)
                    {
                        const bool mir = GH && L.hmirror[0] && X.x0 - 1 == L.hghost[0];
                        const bool neg = mir && L.hmirror[0] < 0, zero = !mir && (wh & kInfoZeroCol);
                        const int v = lane < TY ? lane : lane - TY;
                        const int o = (v + 1) * BX + XOFF - (mir ? 0 : 1);  // column x0 - 1 (x0: mirrored)
                        const T h = zero ? T(0) : lane < TY ? hz(o) : hy(o);
                        X.hn_at(rn, lane < TY ? 2 : 1, v + 1, XOFF - 1) = neg ? -h : h;
                    }
                };
                if constexpr (sizeof(T) == 8)
                {
                    if (unit_dx) fast_h_halo(std::true_type{});
                    else fast_h_halo(std::false_type{});
                }
                else
                    fast_h_halo(std::false_type{});
                }
            }
            else
            {
                auto general_h_own = [&](auto unit) {
                    constexpr bool U = decltype(unit)::value;
                    if (lean_h)
                    {
                        auto lean = [&](auto ax) {
                            constexpr int A = decltype(ax)::value;
#pragma unroll
                            for (int r = 0; r < RPT; ++r)
#pragma unroll
                                for (int p = 0; p < NPT; ++p)
                                    h_own_general<T, PML, false, U, A>(X, q, r0 + r, ol * NPT + p, eA, eB, hA, rn, 63u, q >= 1, true,
                                                                  false, false, idx + r * sy + p, ph[r][p]);
                        };
                        // fp64: a tile plane with CPML along one axis only
                        // takes a copy without the other axes' terms
                        if constexpr (kAxisSpec<T>)
                        {
                            const int ax = ax_h | (X.tab(2, 1)[q].active() ? 4 : 0);
                            if (ax == 1) lean(std::integral_constant<int, 1>{});
                            else if (ax == 2) lean(std::integral_constant<int, 2>{});
                            else if (ax == 4) lean(std::integral_constant<int, 4>{});
#if FFIP_FUSED_F64_AXIS_PAIRS
                            else if (ax == 3) lean(std::integral_constant<int, 3>{});
                            else if (ax == 5) lean(std::integral_constant<int, 5>{});
                            else if (ax == 6) lean(std::integral_constant<int, 6>{});
#endif
                            else lean(std::integral_constant<int, 7>{});
                        }
                        else
                            lean(std::integral_constant<int, 7>{});
                    }
                    else
                    {
#pragma unroll
                        for (int r = 0; r < RPT; ++r)
#pragma unroll
                            for (int p = 0; p < NPT; ++p)
                                h_own_general<T, PML, true, U>(X, q, r0 + r, ol * NPT + p, eA, eB, hA, rn,
                                                          vxy[r][p] & (wh >> kInfoZValidShift), q >= 1, pml_h, h_slots, dft_h,
                                                          idx + r * sy + p, ph[r][p]);
                    }
                };
                if constexpr (sizeof(T) == 8)
                {
                    if (unit_dx) general_h_own(std::true_type{});
                    else general_h_own(std::false_type{});
                }
                else
                    general_h_own(std::false_type{});
                general_halo();
            }
        }
        mbar_arrive(&hd[q & 3]);
        // STGH: copy the H-side psi of the next iteration's own points (read
        // above once this copy's group has completed)
        if (STGH)
        {
            const int q1 = q + 1;
            const unsigned wh1 = q1 <= NP - 2 ? info[q1] : 0u;
            if (q1 <= NP - 2 && !(wh1 & kInfoFastH) && pml_tables && (wh1 & kInfoZPml))
            {
                const bool cz = X.tab(2, 1)[q1].nz();
#pragma unroll
                for (int r = 0; r < RPT; ++r)
#pragma unroll
                    for (int p = 0; p < NPT; ++p)
                    {
                        const bool ch[3] = {X.tab(0, 1)[ol * NPT + p + 1].nz(), X.tab(1, 1)[r0 + r + 1].nz(), cz};
                        const unsigned vb = vxy[r][p] & (wh1 >> kInfoZValidShift);
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                        {
                            const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
                            const bool vh = (vb >> (3 + c)) & 1u;
                            if (vh && ch[a1]) cp_async_elem(stage_slot_h(r, p, c, 0), F.psih_in[c][0] + idx + sz + r * sy + p);
                            if (vh && ch[a2]) cp_async_elem(stage_slot_h(r, p, c, 1), F.psih_in[c][1] + idx + sz + r * sy + p);
                        }
                    }
            }
            cp_async_commit();
        }
        // 2. E(k-1) on the tile from H(k-1) and H(k-2)
        if (do_e)
        {
            // split warps: a warp without CPML on a lean CPML plane takes
            // the plain path (no slots on lean planes)
            const bool warp_fast_e = WFAST && lean_e && warp_plain && !X.tab(2, 0)[q - 1].nz();
            if (fast_e || warp_fast_e)
            {
                auto fast_e_own = [&](auto unit, auto slotted) {
                    constexpr bool U = decltype(unit)::value;
                    constexpr bool SL = decltype(slotted)::value;
                    const T *eS0 = X.e_tile(eS, 0) + offE, *eS1 = X.e_tile(eS, 1) + offE, *eS2 = X.e_tile(eS, 2) + offE;
                    const T *n0 = X.hn_plane(rp, 0) + offN, *n1 = X.hn_plane(rp, 1) + offN, *n2 = X.hn_plane(rp, 2) + offN;
                    const T *p0 = X.hn_plane(rpp, 0) + offN, *p1 = X.hn_plane(rpp, 1) + offN;
                    Vals<T, NPT> hz[RPT + 1], hx[RPT + 1];  // rows r0-1 .. r0+RPT-1
#pragma unroll
                    for (int r = 0; r <= RPT; ++r)
                    {
                        hz[r] = ldv<NPT>(n2 + (r - 1) * RW);
                        hx[r] = ldv<NPT>(n0 + (r - 1) * RW);
                    }
#pragma unroll
                    for (int r = 0; r < RPT; ++r)
                    {
                        const Vals<T, NPT> hyr = ldv<NPT>(n1 + r * RW), hyp = ldv<NPT>(p1 + r * RW), hxp = ldv<NPT>(p0 + r * RW);
                        const Vals<T, NPT> e0 = ldv<NPT>(eS0 + r * BX), e1 = ldv<NPT>(eS1 + r * BX), e2 = ldv<NPT>(eS2 + r * BX);
                        // x - 1 neighbours: the previous point of the pair, or
                        // the previous lane's last point (warp shuffle; the
                        // first lane reads the ring's halo column)
                        T hzw, hyw;
                        if constexpr (SHFL)
                        {
                            hzw = __shfl_up_sync(0xffffffffu, hz[r + 1][NPT - 1], 1);
                            hyw = __shfl_up_sync(0xffffffffu, hyr[NPT - 1], 1);
                            if (lane == 0)
                            {
                                hzw = n2[r * RW - 1];
                                hyw = n1[r * RW - 1];
                            }
                        }
                        else
                        {
                            hzw = n2[r * RW - 1];
                            hyw = n1[r * RW - 1];
                        }
                        Vals<T, NPT> ex, ey, ez;
#pragma unroll
                        for (int p = 0; p < NPT; ++p)
                        {
                            const T hzx = p > 0 ? hz[r + 1][p - 1] : hzw, hyx = p > 0 ? hyr[p - 1] : hyw;
                            ex[p] = e0[p] + coefE * curl_diff<U>(hz[r + 1][p], hz[r][p], hyr[p], hyp[p], ide);
                            ey[p] = e1[p] + coefE * curl_diff<U>(hx[r + 1][p], hxp[p], hz[r + 1][p], hzx, ide);
                            ez[p] = e2[p] + coefE * curl_diff<U>(hyr[p], hyx, hx[r + 1][p], hx[r][p], ide);
                        }
                        // SL: the points with a material slot take the slot's
                        // update from the same curl terms (as the general path)
                        T vds[3][NPT];
                        if constexpr (SL)
                        {
#pragma unroll
                            for (int p = 0; p < NPT; ++p)
                            {
                                vds[0][p] = PE.g_def * ex[p];
                                vds[1][p] = PE.g_def * ey[p];
                                vds[2][p] = PE.g_def * ez[p];
                            }
#pragma unroll
                            for (int p = 0; p < NPT; ++p)
                            {
                                const T hzx = p > 0 ? hz[r + 1][p - 1] : hzw, hyx = p > 0 ? hyr[p - 1] : hyw;
                                if (sl_e[r][p][0] >= 0)
                                    ex[p] = material_rec(PE, PE.slot[0], sl_e[r][p][0], e0[p],
                                                         curl_diff<U>(hz[r + 1][p], hz[r][p], hyr[p], hyp[p], ide), &vds[0][p]);
                                if (sl_e[r][p][1] >= 0)
                                    ey[p] = material_rec(PE, PE.slot[1], sl_e[r][p][1], e1[p],
                                                         curl_diff<U>(hx[r + 1][p], hxp[p], hz[r + 1][p], hzx, ide), &vds[1][p]);
                                if (sl_e[r][p][2] >= 0)
                                    ez[p] = material_rec(PE, PE.slot[2], sl_e[r][p][2], e2[p],
                                                         curl_diff<U>(hyr[p], hyx, hx[r + 1][p], hx[r][p], ide), &vds[2][p]);
                            }
                        }
                        // GH: points left to the face kernel are neither stored
                        // nor summed (they add zero to the DFT sums)
                        unsigned dmr = 0;
#pragma unroll
                        for (int p = 0; p < NPT; ++p) dmr |= dm[r][p];
                        if (!GH || dmr == 0)
                        {
                            st_outv(&F.eout[0][idx_e + r * sy], ex);
                            st_outv(&F.eout[1][idx_e + r * sy], ey);
                            st_outv(&F.eout[2][idx_e + r * sy], ez);
                        }
                        else
                        {
#pragma unroll
                            for (int p = 0; p < NPT; ++p)
                            {
                                if (!(dm[r][p] & 1u)) st_out(&F.eout[0][idx_e + r * sy + p], ex[p]);
                                if (!(dm[r][p] & 2u)) st_out(&F.eout[1][idx_e + r * sy + p], ey[p]);
                                if (!(dm[r][p] & 4u)) st_out(&F.eout[2][idx_e + r * sy + p], ez[p]);
                            }
                        }
                        if (dft_e)
                            for (int c = 0; c < 3; ++c)
                            {
                                const Vals<T, NPT> &ev = c == 0 ? ex : c == 1 ? ey : ez;
                                double v[NPT], vd[NPT];
#pragma unroll
                                for (int p = 0; p < NPT; ++p)
                                {
                                    v[p] = (double)ev[p];
                                    if constexpr (SL)
                                        vd[p] = (double)vds[c][p];
                                    else
                                        vd[p] = (double)(PE.g_def * ev[p]);
                                    if (GH && ((dm[r][p] >> c) & 1u)) v[p] = vd[p] = 0.0;
                                }
                                if constexpr (PML || NPT == 1)
                                {
                                    for (int p = 0; p < NPT; ++p)
                                        if (!GH || !((dm[r][p] >> c) & 1u))
                                            dft_point<T>(PE.nunits, PE.units, PE.phase, c, x + p, X.y0 + r0 + r, k - 1, v[p], vd[p]);
                                }
                                else
                                    dft_points<NPT>(PE.nunits, PE.units, PE.phase, c, x, X.y0 + r0 + r, k - 1, v, vd);
                            }
                    }
                };
                if constexpr (sizeof(T) == 8)
                {
                    if (unit_dx) fast_e_own(std::true_type{}, std::false_type{});
                    else fast_e_own(std::false_type{}, std::false_type{});
                }
                else if (fast_e_sl)
                    fast_e_own(std::false_type{}, std::true_type{});
                else
                    fast_e_own(std::false_type{}, std::false_type{});
            }
            else
            {
                if (STG && pml_e)
                {
                    // this iteration's E psi (STGH: the next iteration's H
                    // psi, committed after it, may stay in flight)
                    if (STGH) cp_async_wait_but_last();
                    else cp_async_wait_all();
                }
                // the interior instance adds the DFT sums of a row's points
                // together, with their loads batched (dft_points)
                constexpr bool DEFER = FFIP_FUSED_DFT_DEFER && !PML && sizeof(T) == 4 && NPT > 1;
                double dv[NPT][3][2];
#pragma unroll
                for (int r = 0; r < RPT; ++r)
                {
#pragma unroll
                    for (int p = 0; p < NPT; ++p)
                    {
                        // staged psi of the own point (stale where the copy was
                        // skipped, i.e. where it is not used)
                        T pe[3][2] = {};
                        if (STG && pml_e)
                        {
#pragma unroll
                            for (int c = 0; c < 3; ++c)
                            {
                                pe[c][0] = *stage_slot(r, p, c, 0);
                                pe[c][1] = *stage_slot(r, p, c, 1);
                            }
                        }
                        const int xi = ol * NPT + p;
                        auto general_e_own = [&](auto unit) {
                            constexpr bool U = decltype(unit)::value;
                            if (lean_e)
                            {
                                auto lean = [&](auto ax) {
                                    constexpr int A = decltype(ax)::value;
                                    e_own_general<T, PML, false, STG, U, A>(X, q - 1, r0 + r, xi, eS, rp, rpp, 63u & ~dm[r][p], true,
                                                                       false, false, idx_e + r * sy + p, sl_e[r][p], pe);
                                };
                                if constexpr (kAxisSpec<T>)
                                {
                                    const int ax = ax_e | (X.tab(2, 0)[q - 1].active() ? 4 : 0);
                                    if (ax == 1) lean(std::integral_constant<int, 1>{});
                                    else if (ax == 2) lean(std::integral_constant<int, 2>{});
                                    else if (ax == 4) lean(std::integral_constant<int, 4>{});
#if FFIP_FUSED_F64_AXIS_PAIRS
                                    else if (ax == 3) lean(std::integral_constant<int, 3>{});
                                    else if (ax == 5) lean(std::integral_constant<int, 5>{});
                                    else if (ax == 6) lean(std::integral_constant<int, 6>{});
#endif
                                    else lean(std::integral_constant<int, 7>{});
                                }
                                else
                                    lean(std::integral_constant<int, 7>{});
                            }
                            else
                                e_own_general<T, PML, true, STG, U>(X, q - 1, r0 + r, xi, eS, rp, rpp,
                                                               vxy[r][p] & (we >> kInfoZValidShift), pml_e, e_slots, dft_e,
                                                               idx_e + r * sy + p, sl_e[r][p], pe,
                                                               DEFER && dft_e ? dv[p] : nullptr);
                        };
                        if constexpr (sizeof(T) == 8)
                        {
                            if (unit_dx) general_e_own(std::true_type{});
                            else general_e_own(std::false_type{});
                        }
                        else
                            general_e_own(std::false_type{});
                    }
                    if (DEFER && dft_e && !lean_e)
                        for (int c = 0; c < 3; ++c)
                        {
                            double v[NPT], vd[NPT];
#pragma unroll
                            for (int p = 0; p < NPT; ++p)
                            {
                                v[p] = dv[p][c][0];
                                vd[p] = dv[p][c][1];
                            }
                            dft_points<NPT>(PE.nunits, PE.units, PE.phase, c, x, X.y0 + r0 + r, k - 1, v, vd);
                        }
                }
            }
        }
        eS = eA;
        eA = eB;
        eB = eB + 1 == SE ? 0 : eB + 1;
        hA = hA + 1 == SHS ? 0 : hA + 1;
        rpp = rp;
        rp = rn;
        rn = (rn + 1) & 3;
    }
    if (STG) cp_async_wait_all();
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

template <typename T, bool IS_E>
__global__ void k_face(const __grid_constant__ FusedLaunch<T> L, const __grid_constant__ FaceList B)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= B.total) return;
    int b = 0;
    while (b + 1 < B.n && t >= B.b[b + 1].start) ++b;
    const FaceBox &X = B.b[b];
    const int64_t u = t - X.start, r = u / X.ni;
    const int i = X.i0 + (int)(u - r * X.ni), j = X.j0 + (int)(r % X.nj), k = X.k0 + (int)(r / X.nj);
    constexpr int C0 = IS_E ? 0 : 3;
    if (X.comp == 0) face_point<T, C0 + 0>(L.fp, i, j, k);
    else if (X.comp == 1) face_point<T, C0 + 1>(L.fp, i, j, k);
    else face_point<T, C0 + 2>(L.fp, i, j, k);
}
} // namespace ffipg
