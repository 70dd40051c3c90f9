// Per-point update rules of the Yee/CPML/ADE/DFT stepper and the parameter
// blocks the kernels take.  The functions are written once, as
// FFIP_HD (host+device) inlines, and called from the CUDA kernels in
// kernels.cu.  Array layout and index conventions: see plan.hpp.
//
// Reference rules restated here (all positions on the reference's doubled
// grid, one array per component here):
//   non-CPML curl   accdb += curl1 - curl2           src/fields.cpp:133-148
//   CPML            phi = b*phi + c*curl;
//                   accdb += phi1 - phi2 + curl1/k1 - curl2/k2
//                                                    src/fields.cpp:89-109
//   H side uses negated strides (-curl E)            src/fields.cpp:174-177
//   constitutive    P_n <- c1 P_n + c2 P'_n + amp c3 E_old;
//                   E = (accdb*dt - sum P_n)/g_inf    src/structure.cpp:56-85
//                   (carried in an equivalent increment form, material_point)
//   DFT             re += cos(2 pi f t) v, im += -sin(2 pi f t) v
//                                                    src/dft.cpp:29-62
// E is carried directly, without the reference's accdb array: for a point
// without poles E += (dt/g_inf) * (curl terms); with poles see material_point.
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define FFIP_HD __host__ __device__ __forceinline__
#define FFIP_HD_CALL __host__ __device__ __noinline__
#define FFIP_UNROLL _Pragma("unroll")
#else
#define FFIP_HD inline
#define FFIP_HD_CALL inline
#define FFIP_UNROLL
#endif

namespace ffipg
{
constexpr int kMaxUnitsPerSide = 24;  // DFT units per side passed to one launch
constexpr int kMaxPhases = 192;       // (unit, frequency) pairs per side
constexpr int kMaxPolesDev = 8;       // must equal kMaxPoles in plan.hpp

struct RowRange
{
    int lo, hi;  // x-index range of slot points in one (j,k) row; lo > hi if none
};

// one slot's constants in one aligned record: dt/g_inf, 1/g_inf, g_inf and
// meta = group + 256 * (poles of the group), an exact small integer
template <typename T>
struct alignas(4 * sizeof(T)) SlotRec
{
    T coef, inv, g, meta;
};

template <typename T>
struct SlotView
{
    const int *map;          // slot index per grid position, -1 = default medium (nullptr: no slots)
    const RowRange *rows;    // per (j,k) row
    const T *g, *coef, *inv; // g_inf, dt/g_inf, 1/g_inf per slot
    const uint8_t *group;    // pole group per slot
    const SlotRec<T> *rec;   // the same per slot, packed
    T *A;                    // pending source sum per slot (H side, slots with poles; else null)
    const T *amp;            // [stride][n]
    T *P, *P1;               // [stride][n] polarisation P and its last increment J = P - P_prev
    // fused pass, H side: the new P / J go to Po / P1o, so that the old ones
    // stay readable for the halo points that neighbouring tiles recompute,
    // and A is left for the engine to clear after the pass; null: in place
    T *Po, *P1o;
    int64_t n;
    int stride;              // poles per slot in amp / P / P1
};

struct DftView
{
    int comp;        // global component 0..5
    int is_db;       // D/B monitor (value = accdb*dt)
    int i0[3], ld[3];
    int nf, foff;    // frequencies and their offset into the phase table
    int64_t npts;
    double *re, *im; // [nf][npts], npts ordered x fastest
};

template <typename T>
struct SideParams
{
    int Mx, My, Mz;
    int64_t sy, sz;
    int vlo[3][3], vhi[3][3];  // own components [c][axis]
    int par[3][3];             // parity of own component c along axis
    T inv_dx, dt;
    T *f[3];                   // own components, read-modify-write
    const T *o[3];             // other side's components, indexed by direction
    T *psi[3][2];              // CPML psi of own component c for its two transverse axes
    const T *pb[3][2], *pc[3][2], *pik[3][2];  // CPML tables [axis][parity], null if no CPML
    T coef_def, g_def;         // default medium: dt/g_inf, g_inf
    SlotView<T> slot[3];
    const uint8_t *grp_np;     // poles per group
    const uint8_t *grp_pool;   // [group][kMaxPolesDev] pool indices
    const T *pool_c;           // [pool][3] = d1, d2, c3 (see material_point)
    int comp_base;             // 0 for E, 3 for H
    int nunits;
    DftView units[kMaxUnitsPerSide];
    double phase[kMaxPhases][2];  // cos(2 pi f t), -sin(2 pi f t)
};

// ---------------------------------------------------------------------------
// DFT accumulation of one point's new value into every matching unit
template <typename T>
FFIP_HD void dft_point(int nunits, const DftView *units, const double (*phase)[2], int gcomp, int i, int j, int k,
                       double v, double vd)
{
    for (int u = 0; u < nunits; ++u)
    {
        const DftView &U = units[u];
        if (U.comp != gcomp) continue;
        int li = i - U.i0[0], lj = j - U.i0[1], lk = k - U.i0[2];
        if ((unsigned)li >= (unsigned)U.ld[0] || (unsigned)lj >= (unsigned)U.ld[1] || (unsigned)lk >= (unsigned)U.ld[2]) continue;
        int64_t l = ((int64_t)lk * U.ld[1] + lj) * U.ld[0] + li;
        double x = U.is_db ? vd : v;
        for (int f = 0; f < U.nf; ++f)
        {
            double cw = phase[U.foff + f][0], sw = phase[U.foff + f][1];
            U.im[f * U.npts + l] += sw * x;
            U.re[f * U.npts + l] += cw * x;
        }
    }
}

// The same for the new values of NPT consecutive x points (i .. i + NPT - 1,
// row j, plane k), as a called function (the plain paths of the fused pass
// call it for tile planes that a unit meets; kept out of line so that its
// registers do not count against the pass's loop).  Per chunk of FC
// frequencies every load of the running sums is issued before the first
// store, so that a thread waits for one round trip per chunk instead of one
// per sum (the arrays may alias as far as the compiler knows); each sum gets
// the same single multiply-add as in dft_point.
#ifndef FFIP_DFT_CHUNK
#define FFIP_DFT_CHUNK 8
#endif
template <int NPT>
FFIP_HD_CALL void dft_points(int nunits, const DftView *units, const double (*phase)[2], int gcomp, int i, int j, int k,
                             const double *v, const double *vd)
{
    constexpr int FC = FFIP_DFT_CHUNK / NPT;
    for (int u = 0; u < nunits; ++u)
    {
        const DftView &U = units[u];
        if (U.comp != gcomp) continue;
        const int lj = j - U.i0[1], lk = k - U.i0[2], li = i - U.i0[0];
        if ((unsigned)lj >= (unsigned)U.ld[1] || (unsigned)lk >= (unsigned)U.ld[2]) continue;
        bool in[NPT];
        bool any = false;
        double x[NPT];
        FFIP_UNROLL
        for (int p = 0; p < NPT; ++p)
        {
            in[p] = (unsigned)(li + p) < (unsigned)U.ld[0];
            any = any || in[p];
            x[p] = U.is_db ? vd[p] : v[p];
        }
        if (!any) continue;
        const int64_t l = ((int64_t)lk * U.ld[1] + lj) * U.ld[0] + li;
        for (int f0 = 0; f0 < U.nf; f0 += FC)
        {
            double re[FC][NPT], im[FC][NPT];
            FFIP_UNROLL
            for (int f = 0; f < FC; ++f)
                FFIP_UNROLL
                for (int p = 0; p < NPT; ++p)
                    if (f0 + f < U.nf && in[p])
                    {
                        im[f][p] = U.im[(f0 + f) * U.npts + l + p];
                        re[f][p] = U.re[(f0 + f) * U.npts + l + p];
                    }
            FFIP_UNROLL
            for (int f = 0; f < FC; ++f)
                FFIP_UNROLL
                for (int p = 0; p < NPT; ++p)
                    if (f0 + f < U.nf && in[p])
                    {
                        const double cw = phase[U.foff + f0 + f][0], sw = phase[U.foff + f0 + f][1];
                        U.im[(f0 + f) * U.npts + l + p] = im[f][p] + sw * x[p];
                        U.re[(f0 + f) * U.npts + l + p] = re[f][p] + cw * x[p];
                    }
        }
    }
}

// Compile-time facts of global component GC (0..5 = Ex Ey Ez Hx Hy Hz): its
// index within its side (= its direction), its two transverse axes (the curl
// derivatives, in the reference's x1 = x3+1, x2 = x3+2 order,
// include/fields.hpp:238-240) and its doubled-grid parities along them.
template <int GC>
struct CompT
{
    static constexpr int c = GC % 3;
    static constexpr int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
    static constexpr int ct = GC == 0 ? 1 : GC == 1 ? 2 : GC == 2 ? 4 : GC == 3 ? 6 : GC == 4 ? 5 : 3;
    static constexpr int q1 = (ct >> a1) & 1, q2 = (ct >> a2) & 1;
};

template <int A>
FFIP_HD int pick(int i, int j, int k)
{
    return A == 0 ? i : (A == 1 ? j : k);
}

// CPML combination at a point where c1 or c2 is non-zero (PML_Stepping::step,
// src/fields.cpp:98-107), from psi values already loaded (psi1/psi2 are not
// used where the matching c is 0).  *ps1/*ps2 receive the new psi.
// fused multiply-add with one rounding, the same on the host and the device
FFIP_HD float fma_rn(float a, float b, float c) { return fmaf(a, b, c); }
FFIP_HD double fma_rn(double a, double b, double c) { return fma(a, b, c); }

// the two halves of the CPML update, roundings fixed (explicit fma) so that
// every code path that forms them gives the same bits: the new psi
// b psi + c curl, and the increment psi1 - psi2 + curl1 / k1 - curl2 / k2
template <typename T>
FFIP_HD T pml_psi(T b, T psi, T cv, T curl)
{
    return fma_rn(cv, curl, b * psi);
}
template <typename T>
FFIP_HD T pml_sum(T p1, T p2, T ik1, T ik2, T curl1, T curl2)
{
    return fma_rn(-curl2, ik2, fma_rn(curl1, ik1, p1 - p2));
}

// n1 / n2: cv1 / cv2 are non-zero (callers that hold these as integer flags
// pass them, and no floating-point compare is issued)
template <typename T>
FFIP_HD T pml_term_nz(bool n1, bool n2, T cv1, T cv2, T b1, T b2, T ik1, T ik2, T curl1, T curl2, T psi1, T psi2, T *ps1,
                      T *ps2)
{
    const T p1 = n1 ? pml_psi(b1, psi1, cv1, curl1) : T(0);
    const T p2 = n2 ? pml_psi(b2, psi2, cv2, curl2) : T(0);
    *ps1 = p1;
    *ps2 = p2;
    return pml_sum(p1, p2, ik1, ik2, curl1, curl2);
}
template <typename T>
FFIP_HD T pml_term(T cv1, T cv2, T b1, T b2, T ik1, T ik2, T curl1, T curl2, T psi1, T psi2, T *ps1, T *ps2)
{
    return pml_term_nz(cv1 != T(0), cv2 != T(0), cv1, cv2, b1, b2, ik1, ik2, curl1, curl2, psi1, psi2, ps1, ps2);
}

// The same with psi read from pin and, when pout is not null, written to pout.
template <typename T>
FFIP_HD T pml_combine_nz(bool n1, bool n2, T cv1, T cv2, T b1, T b2, T ik1, T ik2, T curl1, T curl2, const T *pin1,
                         const T *pin2, T *pout1, T *pout2, int64_t idx)
{
    const T psi1 = n1 ? pin1[idx] : T(0);
    const T psi2 = n2 ? pin2[idx] : T(0);
    T ps1, ps2;
    const T t = pml_term_nz(n1, n2, cv1, cv2, b1, b2, ik1, ik2, curl1, curl2, psi1, psi2, &ps1, &ps2);
    if (n1 && pout1) pout1[idx] = ps1;
    if (n2 && pout2) pout2[idx] = ps2;
    return t;
}
template <typename T>
FFIP_HD T pml_combine(T cv1, T cv2, T b1, T b2, T ik1, T ik2, T curl1, T curl2, const T *pin1, const T *pin2, T *pout1,
                      T *pout2, int64_t idx)
{
    return pml_combine_nz(cv1 != T(0), cv2 != T(0), cv1, cv2, b1, b2, ik1, ik2, curl1, curl2, pin1, pin2, pout1, pout2, idx);
}

// curl increment of accdb at a point, CPML tables read from global memory
template <typename T, int GC>
FFIP_HD T curl_term_global(const SideParams<T> &p, int i, int j, int k, int64_t idx, T curl1, T curl2, const T *pin1,
                           const T *pin2, T *pout1, T *pout2)
{
    using C = CompT<GC>;
    if (p.pc[0][0] == nullptr) return curl1 - curl2;
    const int i1 = pick<C::a1>(i, j, k), i2 = pick<C::a2>(i, j, k);
    const T cv1 = p.pc[C::a1][C::q1][i1], cv2 = p.pc[C::a2][C::q2][i2];
    if (cv1 == T(0) && cv2 == T(0)) return curl1 - curl2;
    return pml_combine(cv1, cv2, p.pb[C::a1][C::q1][i1], p.pb[C::a2][C::q2][i2], p.pik[C::a1][C::q1][i1],
                       p.pik[C::a2][C::q2][i2], curl1, curl2, pin1, pin2, pout1, pout2, idx);
}

// slot index of a point (-1: default medium)
template <typename T>
FFIP_HD int slot_of(const SlotView<T> &S, int My, int i, int j, int k, int64_t idx)
{
    if (!S.map) return -1;
    const RowRange r = S.rows[j + (int64_t)k * My];
    return (i >= r.lo && i <= r.hi) ? S.map[idx] : -1;
}

// one pole of the (P, J) update: J_new = d1 P + d2 J + amp c3 E_old, with
// its roundings fixed (explicit fma), so that every kernel that updates a
// pole gives the same bits
template <typename T>
FFIP_HD T pole_increment(T d1, T d2, T c3, T P, T J, T amp, T old)
{
    return fma_rn(d1, P, fma_rn(d2, J, (amp * c3) * old));
}

// E_new = E_old + ((term + pend) dt - sum J_new) / g_inf, roundings fixed
template <typename T>
FFIP_HD T pole_field(T old, T term, T pend, T dt, T dsum, T inv)
{
    return fma_rn(fma_rn(term + pend, dt, -dsum), inv, old);
}

// Constitutive update of one point given its accdb increment `term`; `old`
// is the point's field before this half step.  Returns the new field; *vd
// receives the D/B value for D/B monitors.  WRITE = false: the same value
// without touching the slot state (a halo point the fused pass recomputes).
template <typename T, bool WRITE = true>
FFIP_HD T material_at(const SideParams<T> &p, const SlotView<T> &S, int slot, T old, T term, T *vd)
{
    T v;
    if (slot < 0)
    {
        v = old + p.coef_def * term;
        *vd = p.g_def * v;
        return v;
    }
    const int g = S.group[slot];
    const int np = p.grp_np[g];
    if (np == 0)
    {
        v = fma_rn(S.coef[slot], term, old);
        *vd = S.g[slot] * v;
        return v;
    }
    // The reference forms E = (accdb*dt - sum P)/g_inf from the running sum
    // accdb.  Its difference between consecutive steps gives the same value
    // without that sum:
    //   E_new = E_old + (dt*(curl terms + sources) - sum (P_new - P_old)) / g_inf,
    // which avoids cancelling two large numbers inside metals (it keeps fp32
    // state accurate) and needs no accdb array.  H-side sources arrive before
    // this update and wait in S.A.
    T pend = T(0);
    if (S.A)
    {
        pend = S.A[slot];
        if (WRITE && !S.Po && pend != T(0)) S.A[slot] = T(0);
    }
    // Each pole keeps P and its last increment J = P - P_prev.  The
    // reference's P_new = c1 P + c2 P_prev + amp c3 E_old is the same as
    //   J_new = d1 P + d2 J + amp c3 E_old,  P_new = P + J_new
    // with d1 = c1 + c2 - 1 and d2 = -c2 (pool_c holds d1, d2, c3), whose
    // inputs are well scaled: for a Drude pole d1 is exactly 0, while c1 ~ 2
    // and c2 ~ -1 lose the small increment in fp32.
    T dsum = T(0), psum = T(0);
    for (int q = 0; q < np; ++q)
    {
        const int pool = p.grp_pool[g * kMaxPolesDev + q];
        const T d1 = p.pool_c[3 * pool], d2 = p.pool_c[3 * pool + 1], c3 = p.pool_c[3 * pool + 2];
        const int64_t s = q * S.n + slot;
        const T Pq = S.P[s], Jq = S.P1[s];
        const T Jn = pole_increment(d1, d2, c3, Pq, Jq, S.amp[s], old);
        const T Pn = Pq + Jn;
        if (WRITE)
        {
            (S.P1o ? S.P1o : S.P1)[s] = Jn;
            (S.Po ? S.Po : S.P)[s] = Pn;
        }
        dsum = dsum + Jn;
        psum = psum + Pn;
    }
    v = pole_field(old, term, pend, p.dt, dsum, S.inv[slot]);
    *vd = fma_rn(S.g[slot], v, psum);  // D = g_inf E + sum P
    return v;
}

// material_at for a slot >= 0 of a side without pending sources (E side),
// from the packed record; the loads of the first two poles do not wait for
// the record, so one memory latency covers the point.  Same arithmetic and
// evaluation order as material_at.
template <typename T>
FFIP_HD T material_rec(const SideParams<T> &p, const SlotView<T> &S, int slot, T old, T term, T *vd)
{
    T P0 = T(0), J0 = T(0), A0 = T(0), P1v = T(0), J1 = T(0), A1 = T(0);
    if (S.stride >= 1)
    {
        P0 = S.P[slot];
        J0 = S.P1[slot];
        A0 = S.amp[slot];
    }
    if (S.stride >= 2)
    {
        P1v = S.P[S.n + slot];
        J1 = S.P1[S.n + slot];
        A1 = S.amp[S.n + slot];
    }
    const SlotRec<T> r = S.rec[slot];
    const int meta = (int)r.meta, g = meta & 255, np = meta >> 8;
    if (np == 0)
    {
        const T v = fma_rn(r.coef, term, old);
        *vd = r.g * v;
        return v;
    }
    T dsum = T(0), psum = T(0);
    for (int q = 0; q < np; ++q)
    {
        const int pool = p.grp_pool[g * kMaxPolesDev + q];
        const T d1 = p.pool_c[3 * pool], d2 = p.pool_c[3 * pool + 1], c3 = p.pool_c[3 * pool + 2];
        const int64_t s = q * S.n + slot;
        const T Pq = q == 0 ? P0 : q == 1 ? P1v : S.P[s];
        const T Jq = q == 0 ? J0 : q == 1 ? J1 : S.P1[s];
        const T Aq = q == 0 ? A0 : q == 1 ? A1 : S.amp[s];
        const T Jn = pole_increment(d1, d2, c3, Pq, Jq, Aq, old);
        const T Pn = Pq + Jn;
        S.P1[s] = Jn;
        S.P[s] = Pn;
        dsum = dsum + Jn;
        psum = psum + Pn;
    }
    const T v = pole_field(old, term, T(0), p.dt, dsum, r.inv);
    *vd = fma_rn(r.g, v, psum);
    return v;
}

// Full update of one point of global component GC (E side: GC < 3), in place,
// reading the other side's fields from p.o.  E reads its odd neighbours at
// index i-1 and i, H (the reference's negated strides, src/fields.cpp:174-177)
// its even neighbours at i and i+1.
template <typename T, int GC>
FFIP_HD void update_point(const SideParams<T> &p, int i, int j, int k)
{
    using C = CompT<GC>;
    constexpr bool IS_E = GC < 3;
    const int64_t idx = (int64_t)i + (int64_t)j * p.sy + (int64_t)k * p.sz;
    const int64_t s1 = C::a1 == 0 ? 1 : (C::a1 == 1 ? p.sy : p.sz);
    const int64_t s2 = C::a2 == 0 ? 1 : (C::a2 == 1 ? p.sy : p.sz);
    const T *O1 = p.o[C::a2];  // derivative along a1 of the other-side component pointing along a2
    const T *O2 = p.o[C::a1];
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
    constexpr int c = C::c;
    const T term = curl_term_global<T, GC>(p, i, j, k, idx, curl1, curl2, p.psi[c][0], p.psi[c][1], p.psi[c][0], p.psi[c][1]);
    const int slot = slot_of(p.slot[c], p.My, i, j, k, idx);
    T vd;
    T *F = p.f[c];
    const T v = material_at(p, p.slot[c], slot, F[idx], term, &vd);
    F[idx] = v;
    if (p.nunits) dft_point<T>(p.nunits, p.units, p.phase, GC, i, j, k, (double)v, (double)vd);
}

// ---------------------------------------------------------------------------
// sources: one thread per distinct source grid point, dipoles summed in the
// reference's list order (src/fields.cpp:17-33)
template <typename T>
struct SourceParams
{
    int npts;
    const uint8_t *comp;      // own-side component 0..2 per point
    const int64_t *lin;
    const int *off;           // CSR into the dipole arrays
    const double *amp, *start, *end, *width;
    const uint8_t *kind;      // 1 Gaussian1, 2 Gaussian2
    double time;
    T dt;
    T *f[3];
    SlotView<T> slot[3];
    T coef_def;
    const uint8_t *grp_np;
    // 1: applied after the side's update (E sources), with the matching DFT
    // correction; 0: applied before the side's update (H sources)
    int correct;
    const int *moff;          // CSR per point into (munit, mlin)
    const int *munit;
    const int64_t *mlin;
    int nunits;
    DftView units[kMaxUnitsPerSide];
    double phase[kMaxPhases][2];
};

// src/utility.cpp:260-272
FFIP_HD double gaussian1(double t, double width)
{
    double arg = (t / width);
    return arg * exp(-arg * arg / 2);
}
FFIP_HD double gaussian2(double t, double width)
{
    double arg = (t / width);
    arg = arg * arg;
    return (1 - arg) * exp(-arg);
}

template <typename T>
FFIP_HD void source_point(const SourceParams<T> &p, int q)
{
    double s = 0.0;
    bool any = false;
    for (int d = p.off[q]; d < p.off[q + 1]; ++d)
    {
        if (!(p.time > p.start[d] && p.time < p.end[d])) continue;
        double mid = (p.start[d] + p.end[d]) / 2;
        double g = p.kind[d] == 1 ? gaussian1(p.time - mid, p.width[d]) : gaussian2(p.time - mid, p.width[d]);
        s = s + p.amp[d] * g;
        any = true;
    }
    if (!any) return;
    const int c = p.comp[q];
    const int64_t idx = p.lin[q];
    const SlotView<T> &S = p.slot[c];
    const int slot = S.map ? S.map[idx] : -1;
    const T sv = (T)s;
    T delta, deltad;
    if (slot >= 0 && p.grp_np[S.group[slot]] > 0)
    {
        // a point with poles: before its update (H sources) the source waits
        // in S.A, because the polarisation update must still see the old
        // field; after its update (E sources) the field follows directly.
        if (!p.correct)
        {
            S.A[slot] = S.A[slot] + sv;
            return;
        }
        delta = sv * p.dt * S.inv[slot];
        deltad = sv * p.dt;
    }
    else
    {
        const T coef = slot >= 0 ? S.coef[slot] : p.coef_def;
        delta = coef * sv;
        deltad = sv * p.dt;
    }
    p.f[c][idx] += delta;
    if (p.correct)
        for (int m = p.moff[q]; m < p.moff[q + 1]; ++m)
        {
            const DftView &U = p.units[p.munit[m]];
            const double x = U.is_db ? (double)deltad : (double)delta;
            for (int f = 0; f < U.nf; ++f)
            {
                U.im[f * U.npts + p.mlin[m]] += p.phase[U.foff + f][1] * x;
                U.re[f * U.npts + p.mlin[m]] += p.phase[U.foff + f][0] * x;
            }
        }
}

// ---------------------------------------------------------------------------
// Flux through a flux region (Flux_Region.get_values, ffip/simulation.py:
// 121-160): at every integration point (x_i, y_j, z_k), the E1 and H2 DFT
// monitors are interpolated linearly over their output grids (the
// reference's Fields_DFT interpolant, ffip/simulation.py:55-91: an axis of
// one point is widened to +-dx/2 with the value repeated), and Re(E1 conj(H2))
// times the point's weight is summed per frequency.
constexpr int kMaxFluxFreqs = 64;
struct FluxGrid
{
    const double *re, *im;    // the monitor unit's sums [unit frequency][local point]
    int64_t npts;
    int ld[3];                // local box dims (points)
    int off[3];               // local box offset within the output grid (points)
    int dim[3];               // output grid dims (points)
    double g0[3], gs[3];      // output grid: coordinate of point i = g0 + i gs (widened axes: 2 points)
    int n[3];                 // grid points per axis for the interpolation (dim, or 2 where widened)
    int wide[3];              // axis widened from one point
    int fidx[kMaxFluxFreqs];  // unit frequency index of each requested frequency
};
struct FluxArgs
{
    FluxGrid e1, h2;
    int nf;
    int n[3];                 // integration points per axis
    const double *x, *y, *z;  // their coordinates
    const double *w;          // their weights, [k][j][i]
};

// scipy's RegularGridInterpolator, linear, along one axis: cell index and
// the distance into it
FFIP_HD void flux_axis(const FluxGrid &G, int a, double q, int &i, double &t)
{
    const int n = G.n[a];
    // searchsorted(grid, q, "left") - 1, clipped to [0, n - 2]
    int lo = 0, hi = n;
    while (lo < hi)
    {
        const int mid = (lo + hi) / 2;
        if (G.g0[a] + mid * G.gs[a] < q) lo = mid + 1;
        else hi = mid;
    }
    i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    const double gi = G.g0[a] + i * G.gs[a], gj = G.g0[a] + (i + 1) * G.gs[a];
    t = (q - gi) / (gj - gi);
}

// value of grid point (ix, iy, iz) of the output grid at unit frequency fi
// (zero outside the unit's local box, as the output assembly leaves it)
FFIP_HD void flux_node(const FluxGrid &G, int fi, int ix, int iy, int iz, double &re, double &im)
{
    const int p[3] = {G.wide[0] ? 0 : ix, G.wide[1] ? 0 : iy, G.wide[2] ? 0 : iz};
    const int l0 = p[0] - G.off[0], l1 = p[1] - G.off[1], l2 = p[2] - G.off[2];
    if (l0 < 0 || l1 < 0 || l2 < 0 || l0 >= G.ld[0] || l1 >= G.ld[1] || l2 >= G.ld[2])
    {
        re = im = 0.0;
        return;
    }
    const int64_t l = ((int64_t)l2 * G.ld[1] + l1) * G.ld[0] + l0;
    re = G.re[fi * G.npts + l];
    im = G.im[fi * G.npts + l];
}

FFIP_HD void flux_interp(const FluxGrid &G, int f, double x, double y, double z, double &re, double &im)
{
    int i[3];
    double t[3];
    flux_axis(G, 0, x, i[0], t[0]);
    flux_axis(G, 1, y, i[1], t[1]);
    flux_axis(G, 2, z, i[2], t[2]);
    re = im = 0.0;
    for (int c = 0; c < 8; ++c)
    {
        const int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
        const double w = (dx ? t[0] : 1 - t[0]) * (dy ? t[1] : 1 - t[1]) * (dz ? t[2] : 1 - t[2]);
        double r, m;
        flux_node(G, G.fidx[f], i[0] + dx, i[1] + dy, i[2] + dz, r, m);
        re += w * r;
        im += w * m;
    }
}

// contribution of integration point t (x fastest) to frequency f
FFIP_HD double flux_point(const FluxArgs &A, int64_t t, int f)
{
    const int i = (int)(t % A.n[0]), j = (int)(t / A.n[0] % A.n[1]), k = (int)(t / ((int64_t)A.n[0] * A.n[1]));
    double er, ei, hr, hi;
    flux_interp(A.e1, f, A.x[i], A.y[j], A.z[k], er, ei);
    flux_interp(A.h2, f, A.x[i], A.y[j], A.z[k], hr, hi);
    return (er * hr + ei * hi) * A.w[t];  // Re(e1 conj(h2)) * weight
}

// ---------------------------------------------------------------------------
// PEC/PMC/periodic ghost planes (Fields::sync_boundary, src/fields.cpp:327-482)
constexpr int kMaxFaces = 36;
struct GhostFace
{
    int comp;     // global component 0..5
    int axis;     // normal axis
    int src, dst; // array index along the axis
    int mult;     // +1 / -1
    int u0, u1;   // first index and count along the first in-plane axis (ghost_axes)
    int v0, v1;   // ... second in-plane axis
};

// In-plane axes of a ghost face: x first where it lies in the plane, so that
// the threads of a warp (along u) write consecutive addresses
FFIP_HD void ghost_axes(int axis, int &au, int &av)
{
    au = axis == 0 ? 1 : 0;
    av = axis == 2 ? 1 : 2;
}
template <typename T>
struct GhostParams
{
    int nfaces;
    int64_t sy, sz;
    T *f[6];
    GhostFace faces[kMaxFaces];
};

template <typename T>
FFIP_HD void ghost_point(const GhostParams<T> &p, int face, int u, int v)
{
    const GhostFace &F = p.faces[face];
    if (u >= F.u1 || v >= F.v1) return;
    const int64_t st[3] = {1, p.sy, p.sz};
    int au, av;
    ghost_axes(F.axis, au, av);
    const int64_t base = (int64_t)(F.u0 + u) * st[au] + (int64_t)(F.v0 + v) * st[av];
    T *A = p.f[F.comp];
    A[base + (int64_t)F.dst * st[F.axis]] = A[base + (int64_t)F.src * st[F.axis]] * (T)F.mult;
}
} // namespace ffipg
