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
#else
#define FFIP_HD inline
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

template <typename T>
struct SlotView
{
    const int *map;          // slot index per grid position, -1 = default medium (nullptr: no slots)
    const RowRange *rows;    // per (j,k) row
    const T *g, *coef, *inv; // g_inf, dt/g_inf, 1/g_inf per slot
    const uint8_t *group;    // pole group per slot
    T *A;                    // pending source sum per slot (H side, slots with poles; else null)
    const T *amp;            // [stride][n]
    T *P, *P1;               // [stride][n] polarisation P and its last increment J = P - P_prev
    int64_t n;
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

// CPML-aware curl combination for one point (returns the increment of accdb).
// psi is read from psi_in and, when psi_out is not null, written to psi_out.
template <typename T>
FFIP_HD T curl_term(const SideParams<T> &p, int c, const int ii[3], int64_t idx, T curl1, T curl2, T *psi_in1,
                    T *psi_in2, T *psi_out1, T *psi_out2)
{
    const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
    if (p.pc[a1][0] == nullptr) return curl1 - curl2;
    const int q1 = p.par[c][a1], q2 = p.par[c][a2];
    const T cv1 = p.pc[a1][q1][ii[a1]], cv2 = p.pc[a2][q2][ii[a2]];
    if (cv1 == T(0) && cv2 == T(0)) return curl1 - curl2;
    T ps1 = T(0), ps2 = T(0);
    if (cv1 != T(0))
    {
        ps1 = p.pb[a1][q1][ii[a1]] * psi_in1[idx] + cv1 * curl1;
        if (psi_out1) psi_out1[idx] = ps1;
    }
    if (cv2 != T(0))
    {
        ps2 = p.pb[a2][q2][ii[a2]] * psi_in2[idx] + cv2 * curl2;
        if (psi_out2) psi_out2[idx] = ps2;
    }
    return ps1 - ps2 + curl1 * p.pik[a1][q1][ii[a1]] - curl2 * p.pik[a2][q2][ii[a2]];
}

// Constitutive update of one point given its curl increment; `old` is the
// point's field before this half step.  Writes the new field to *out and
// returns it; *vd receives the D/B value for D/B monitors.
template <typename T>
FFIP_HD T material_point(const SideParams<T> &p, int c, int i, int j, int k, int64_t idx, T old, T term, T *out, T *vd)
{
    const SlotView<T> &S = p.slot[c];
    int slot = -1;
    if (S.map)
    {
        RowRange r = S.rows[j + (int64_t)k * p.My];
        if (i >= r.lo && i <= r.hi) slot = S.map[idx];
    }
    T v;
    if (slot < 0)
    {
        v = old + p.coef_def * term;
        *vd = p.g_def * v;
    }
    else
    {
        const int g = S.group[slot];
        const int np = p.grp_np[g];
        if (np == 0)
        {
            v = old + S.coef[slot] * term;
            *vd = S.g[slot] * v;
        }
        else
        {
            // The reference forms E = (accdb*dt - sum P)/g_inf from the running
            // sum accdb.  Its difference between consecutive steps gives the
            // same value without that sum:
            //   E_new = E_old + (dt*(curl terms + sources) - sum (P_new - P_old)) / g_inf,
            // which avoids cancelling two large numbers inside metals (it
            // keeps fp32 state accurate) and needs no accdb array.  H-side
            // sources arrive before this update and wait in S.A.
            T pend = T(0);
            if (S.A)
            {
                pend = S.A[slot];
                if (pend != T(0)) S.A[slot] = T(0);
            }
            // Each pole keeps P and its last increment J = P - P_prev.  The
            // reference's P_new = c1 P + c2 P_prev + amp c3 E_old is the same as
            //   J_new = d1 P + d2 J + amp c3 E_old,  P_new = P + J_new
            // with d1 = c1 + c2 - 1 and d2 = -c2 (pool_c holds d1, d2, c3),
            // whose inputs are well scaled: for a Drude pole d1 is exactly 0,
            // while c1 ~ 2 and c2 ~ -1 lose the small increment in fp32.
            T dsum = T(0), psum = T(0);
            for (int q = 0; q < np; ++q)
            {
                const int pool = p.grp_pool[g * kMaxPolesDev + q];
                const T d1 = p.pool_c[3 * pool], d2 = p.pool_c[3 * pool + 1], c3 = p.pool_c[3 * pool + 2];
                const int64_t s = q * S.n + slot;
                const T Pq = S.P[s], Jq = S.P1[s];
                const T Jn = d1 * Pq + d2 * Jq + S.amp[s] * c3 * old;
                const T Pn = Pq + Jn;
                S.P1[s] = Jn;
                S.P[s] = Pn;
                dsum = dsum + Jn;
                psum = psum + Pn;
            }
            v = old + ((term + pend) * p.dt - dsum) * S.inv[slot];
            *vd = S.g[slot] * v + psum;  // D = g_inf E + sum P
        }
    }
    *out = v;
    return v;
}

// Full update of one point of own component c on side E (IS_E) or H, in
// place, reading the other side's fields from p.o.
template <typename T, bool IS_E>
FFIP_HD void update_point(const SideParams<T> &p, int c, int i, int j, int k)
{
    const int64_t idx = (int64_t)i + (int64_t)j * p.sy + (int64_t)k * p.sz;
    const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
    const int64_t st[3] = {1, p.sy, p.sz};
    const T *O1 = p.o[a2];  // derivative along a1 of the other-side component pointing along a2
    const T *O2 = p.o[a1];
    T curl1, curl2;
    if (IS_E)
    {
        curl1 = (O1[idx] - O1[idx - st[a1]]) * p.inv_dx;
        curl2 = (O2[idx] - O2[idx - st[a2]]) * p.inv_dx;
    }
    else
    {
        curl1 = (O1[idx] - O1[idx + st[a1]]) * p.inv_dx;
        curl2 = (O2[idx] - O2[idx + st[a2]]) * p.inv_dx;
    }
    const int ii[3] = {i, j, k};
    T term = curl_term(p, c, ii, idx, curl1, curl2, p.psi[c][0], p.psi[c][1], p.psi[c][0], p.psi[c][1]);
    T vd;
    T *F = p.f[c];
    T v = material_point(p, c, i, j, k, idx, F[idx], term, &F[idx], &vd);
    if (p.nunits) dft_point<T>(p.nunits, p.units, p.phase, p.comp_base + c, i, j, k, (double)v, (double)vd);
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
// PEC/PMC/periodic ghost planes (Fields::sync_boundary, src/fields.cpp:327-482)
constexpr int kMaxFaces = 36;
struct GhostFace
{
    int comp;     // global component 0..5
    int axis;     // normal axis
    int src, dst; // array index along the axis
    int mult;     // +1 / -1
    int u0, u1;   // first index and count along the first in-plane axis
    int v0, v1;   // ... second in-plane axis
};
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
    const int au = (F.axis + 1) % 3, av = (F.axis + 2) % 3;
    const int64_t base = (int64_t)(F.u0 + u) * st[au] + (int64_t)(F.v0 + v) * st[av];
    T *A = p.f[F.comp];
    A[base + (int64_t)F.dst * st[F.axis]] = A[base + (int64_t)F.src * st[F.axis]] * (T)F.mult;
}
} // namespace ffipg
