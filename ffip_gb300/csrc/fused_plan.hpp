// Host side of the fused pass: the split of a time step's points (which
// points the pass owns, which the face kernel updates as a list of boxes,
// which PEC / PMC faces the pass mirrors into the halo of its first tiles)
// and the pass's CTA job lists.  Plain C++ (no CUDA), shared by the CUDA
// backend and the host tests.
#pragma once
#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <utility>
#include <vector>

#include "stencil.cuh"

namespace ffipg
{
// The points of one side that the pass does not own, as boxes of one
// component each: x >= xlim or y >= ylim, and for E the layers whose curl
// reads a deferred H ghost
struct FaceBox
{
    int comp;       // component of the side, 0..2
    int i0, ni;     // x range
    int j0, nj;     // y range
    int k0;         // first z plane (the box's count follows from the next start)
    int64_t start;  // index of the box's first point in the list
};
constexpr int kMaxFaceBoxes = 18;  // 3 components x 6 sides of a box difference
struct FaceList
{
    int n;
    int64_t total;
    FaceBox b[kMaxFaceBoxes];
};

// x / y extents the pass's tiles cover (1 <= y < ylim, first_x <= x < xlim):
// a whole number of tiles (tx columns, ty rows) unless the valid extent is
// one or two points more, which go to the face kernel instead of a nearly
// empty tile
inline void fused_limits(int xend, int yend, int first_x, int tx, int ty, int &nbx, int &nby, int &xlim, int &ylim)
{
    const int nxp = xend - first_x, nyp = yend - 1;
    const int rx = nxp % tx, ry = nyp % ty;
    nbx = (nxp >= tx && rx <= 2) ? nxp / tx : (nxp + tx - 1) / tx;
    nby = (nyp >= ty && ry <= 2) ? nyp / ty : (nyp + ty - 1) / ty;
    xlim = std::min(xend, first_x + nbx * tx);
    ylim = std::min(yend, 1 + nby * ty);
}

struct FusedOwnership
{
    int elo[3][3], ehi[3][3];  // E points the pass owns, per component and axis
    int hmirror[2], hghost[2]; // PEC / PMC low x / y face mirrored into the halo (0: none)
};

// E points the pass owns: the valid range less the layers whose curl reads
// an H ghost plane of `faces` (E component c reads H component (c + 2) % 3
// along axis (c + 1) % 3 and (c + 1) % 3 along (c + 2) % 3, at its own index
// and the one below; ghost planes lie outside the valid H range, so those
// layers are the first / last of the range).  mirror: a PEC / PMC face at
// the low x / y end whose ghost is the column / row just before the first
// tile (the ghost mirrors the index after it) is mirrored into the halo of
// the tiles there instead, and its E layer stays owned.
inline FusedOwnership fused_ownership(const int evlo[3][3], const int evhi[3][3], const GhostFace *faces, int nfaces, int first_x,
                                      bool mirror)
{
    FusedOwnership o;
    for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 3; ++a)
        {
            o.elo[c][a] = evlo[c][a];
            o.ehi[c][a] = evhi[c][a];
        }
    const int first[2] = {first_x, 1};
    for (int a = 0; a < 2; ++a)
    {
        o.hmirror[a] = 0;
        o.hghost[a] = -1;
    }
    auto mirrorable = [&](const GhostFace &G) {
        return mirror && G.comp >= 3 && G.axis < 2 && G.dst == first[G.axis] - 1 && G.src == G.dst + 1;
    };
    for (int f = 0; f < nfaces; ++f)
        if (mirrorable(faces[f]))
        {
            o.hmirror[faces[f].axis] = faces[f].mult;
            o.hghost[faces[f].axis] = faces[f].dst;
        }
    for (int f = 0; f < nfaces; ++f)
    {
        const GhostFace &G = faces[f];
        if (G.comp < 3 || mirrorable(G)) continue;
        const int ch = G.comp - 3, a = G.axis;
        for (int c = 0; c < 3; ++c)
        {
            if (!((ch == (c + 2) % 3 && a == (c + 1) % 3) || (ch == (c + 1) % 3 && a == (c + 2) % 3))) continue;
            for (int i = G.dst; i <= G.dst + 1; ++i)
            {
                int &lo = o.elo[c][a], &hi = o.ehi[c][a];
                if (i < lo || i > hi) continue;
                if (i == lo) ++lo;
                else if (i == hi) --hi;
                else throw std::runtime_error("fused pass: a ghost plane inside the grid");
            }
        }
    }
    return o;
}

// The valid points of one side's components that the pass does not own, as
// disjoint boxes: the valid range V less the owned box W (x < xlim, y <
// ylim and, where given, the range lo_own .. hi_own), cut along x, then y,
// then z
inline FaceList fused_face_list(const int vlo[3][3], const int vhi[3][3], const int (*lo_own)[3], const int (*hi_own)[3], int xlim,
                                int ylim)
{
    FaceList B{};
    for (int c = 0; c < 3; ++c)
    {
        int v0[3], v1[3], w0[3], w1[3];
        bool vempty = false, wempty = false;
        for (int a = 0; a < 3; ++a)
        {
            v0[a] = vlo[c][a];
            v1[a] = vhi[c][a];
            w0[a] = lo_own ? std::max(v0[a], lo_own[c][a]) : v0[a];
            w1[a] = hi_own ? std::min(v1[a], hi_own[c][a]) : v1[a];
            if (a == 0) w1[a] = std::min(w1[a], xlim - 1);
            if (a == 1) w1[a] = std::min(w1[a], ylim - 1);
            vempty = vempty || v1[a] < v0[a];
            wempty = wempty || w1[a] < w0[a];
        }
        if (vempty) continue;
        auto add = [&](const int (&b0)[3], const int (&b1)[3]) {
            if (B.n == kMaxFaceBoxes) throw std::runtime_error("fused pass: too many face boxes");
            FaceBox &X = B.b[B.n++];
            X.comp = c;
            X.i0 = b0[0];
            X.ni = b1[0] - b0[0] + 1;
            X.j0 = b0[1];
            X.nj = b1[1] - b0[1] + 1;
            X.k0 = b0[2];
            X.start = B.total;
            B.total += (int64_t)X.ni * X.nj * (b1[2] - b0[2] + 1);
        };
        if (wempty)
        {
            add(v0, v1);
            continue;
        }
        int lo[3] = {v0[0], v0[1], v0[2]}, hi[3] = {v1[0], v1[1], v1[2]};
        for (int a = 0; a < 3; ++a)
        {
            if (w0[a] > lo[a])
            {
                int b0[3] = {lo[0], lo[1], lo[2]}, b1[3] = {hi[0], hi[1], hi[2]};
                b1[a] = w0[a] - 1;
                add(b0, b1);
            }
            if (w1[a] < hi[a])
            {
                int b0[3] = {lo[0], lo[1], lo[2]}, b1[3] = {hi[0], hi[1], hi[2]};
                b0[a] = w1[a] + 1;
                add(b0, b1);
            }
            lo[a] = w0[a];
            hi[a] = w1[a];
        }
    }
    return B;
}

// CTA jobs of the pass: tile origin (x, y) and owned z planes [z, w)
struct JobBox
{
    int x, y, z, w;
};
// a DFT monitor unit's local box (array indices) and its frequencies
struct DftBox
{
    int i0[3], ld[3], nf;
};
struct JobInputs
{
    std::vector<char> pml[3];         // CPML (c != 0 at either parity) per position along each axis
    std::vector<RowRange> rows[3];    // E material slot row ranges per (j, k), empty: no slots
    std::vector<DftBox> dft;          // E and H monitor units
    int My = 0, Mz = 0;
    int xlim = 0, ylim = 0, kbeg = 0, kend = 0;
    int nbx = 0, nby = 0;             // x units of TXP columns, y tiles of TY rows
    int TX = 0, TXP = 0, TY = 0, KCH = 0;
};
struct JobLists
{
    std::vector<JobBox> b, in;  // CPML instance jobs, then interior instance jobs
    // no interior job holds the last x tile or the last y tile: the tiles
    // whose new H the E half of the face kernel reads all belong to the
    // CPML instance
    bool face_in_pml = true;
};

// The jobs of the pass (the CUDA backend builds them once per grid, CPML
// tables and media): x is cut into units of TXP columns from first_x; a
// unit, row of tiles and z chunk without any CPML point in the unit with its
// low-x halo (nor in the row or the chunk) may go to the instance without
// CPML code, TX / TXP adjacent such units per job; z chunks of at most KCH
// planes, the longest CPML-free run of planes chunked apart from the rest.
// slots_to_p: units whose rows hold E material slots go to the CPML
// instance; dft_split > 0: a job whose planes meet DFT monitors is split
// along z into 1 + (frequencies summed over the monitors it meets) /
// dft_split pieces; heavy_first: within each instance the jobs with DFT sums
// (then those with slots) go first; cpml_order: then by the number of axes
// along which the job meets CPML.
inline JobLists fused_jobs(const JobInputs &I, int first_x, bool slots_to_p, int dft_split, bool heavy_first, bool cpml_order)
{
    const int TX = I.TX, TXP = I.TXP, TY = I.TY, KCH = I.KCH;
    auto any = [&](int a, int lo, int hi) {  // CPML anywhere in [lo, hi]
        const int len = (int)I.pml[a].size();
        for (int i = std::max(lo, 0); i <= std::min(hi, len - 1); ++i)
            if (I.pml[a][i]) return true;
        return false;
    };
    // z: chunks [a, b) whose planes a-1 .. b-1 hold no CPML point come from
    // the longest run f0 .. f1 of such planes (a = f0 + 1, b = f1 + 1),
    // chunked apart from the rest
    int za = I.kbeg, zb = I.kbeg;
    for (int f = I.kbeg - 1; f < I.kend;)
    {
        int e = f;
        while (e < I.kend && !any(2, e, e)) ++e;  // planes f .. e-1 are free
        const int a = std::max(f + 1, I.kbeg), bnd = std::min(e, I.kend);
        if (bnd - a > zb - za)
        {
            za = a;
            zb = bnd;
        }
        f = e + 1;
    }
    std::vector<std::pair<int, int>> chunks;
    auto split = [&](int lo, int hi) {
        if (hi <= lo) return;
        const int nch = (hi - lo + KCH - 1) / KCH;
        for (int i = 0; i < nch; ++i)
            chunks.emplace_back(lo + (int)((int64_t)(hi - lo) * i / nch), lo + (int)((int64_t)(hi - lo) * (i + 1) / nch));
    };
    split(I.kbeg, za);
    split(za, zb);
    split(zb, I.kend);
    auto meets = [&](const DftBox &U, const JobBox &j, int tx) {
        return U.i0[0] < j.x + tx && U.i0[0] + U.ld[0] > j.x && U.i0[1] < j.y + TY && U.i0[1] + U.ld[1] > j.y && U.i0[2] < j.w &&
               U.i0[2] + U.ld[2] > j.z - 1;
    };
    // 2: a DFT unit meets the job's box, 1: material slots in its rows
    auto heavy = [&](const JobBox &j, int tx) {
        int w = 0;
        for (const DftBox &U : I.dft)
            if (meets(U, j, tx)) w = 2;
        for (int c = 0; c < 3 && w < 1; ++c)
            for (int k = std::max(j.z - 1, 0); k < std::min(j.w, I.Mz) && w < 1 && !I.rows[c].empty(); ++k)
                for (int y = j.y; y < std::min(j.y + TY, I.My); ++y)
                {
                    const RowRange &rr = I.rows[c][(size_t)k * I.My + y];
                    if (rr.lo <= rr.hi && rr.lo < j.x + tx && rr.hi >= j.x)
                    {
                        w = 1;
                        break;
                    }
                }
        return w;
    };
    JobLists J;
    for (auto &ch : chunks)
    {
        const bool zin = !any(2, ch.first - 1, ch.second - 1);
        for (int by = 0; by < std::max(I.nby, 1); ++by)
        {
            const int y0 = 1 + by * TY;
            const bool yin = !any(1, y0 - 1, y0 + TY - 1);
            const int nu = std::max(I.nbx, 1), per = TX / TXP;
            std::vector<char> plain(nu);
            for (int u = 0; u < nu; ++u)
            {
                const int x0 = first_x + u * TXP;
                plain[u] = zin && yin && !any(0, x0 - 1, x0 + TXP - 1) &&
                           !(slots_to_p && heavy(JobBox{x0, y0, ch.first, ch.second}, TXP) == 1);
            }
            for (int u = 0; u < nu;)
            {
                const int x0 = first_x + u * TXP;
                bool all = u + per <= nu;
                for (int t = 0; t < per && all; ++t) all = plain[u + t] != 0;
                if (all)
                {
                    J.in.push_back(JobBox{x0, y0, ch.first, ch.second});
                    u += per;
                }
                else
                {
                    if (x0 < I.xlim) J.b.push_back(JobBox{x0, y0, ch.first, ch.second});
                    ++u;
                }
            }
        }
    }
    if (dft_split > 0)
    {
        auto split_dft = [&](std::vector<JobBox> &v, int tx) {
            std::vector<JobBox> o;
            o.reserve(v.size());
            for (const JobBox &j : v)
            {
                int nf = 0;
                for (const DftBox &U : I.dft)
                    if (meets(U, j, tx)) nf += U.nf;
                const int planes = j.w - j.z;
                const int m = nf ? std::max(1, std::min(planes, 1 + nf / dft_split)) : 1;
                for (int i = 0; i < m; ++i)
                    o.push_back(JobBox{j.x, j.y, j.z + (int)((int64_t)planes * i / m), j.z + (int)((int64_t)planes * (i + 1) / m)});
            }
            v.swap(o);
        };
        split_dft(J.b, TXP);
        split_dft(J.in, TX);
    }
    if (heavy_first)
    {
        auto cpml_axes = [&](const JobBox &j, int tx) {
            return (int)any(0, j.x - 1, j.x + tx - 1) + (int)any(1, j.y - 1, j.y + TY - 1) + (int)any(2, j.z - 1, j.w - 1);
        };
        auto order = [&](std::vector<JobBox> &v, int tx) {
            std::vector<std::pair<int, size_t>> key(v.size());
            for (size_t i = 0; i < v.size(); ++i) key[i] = {-(4 * heavy(v[i], tx) + (cpml_order ? cpml_axes(v[i], tx) : 0)), i};
            std::stable_sort(key.begin(), key.end());
            std::vector<JobBox> o(v.size());
            for (size_t i = 0; i < v.size(); ++i) o[i] = v[key[i].second];
            v.swap(o);
        };
        order(J.b, TXP);
        order(J.in, TX);
    }
    for (const JobBox &j : J.in)
        if (j.x + TX >= I.xlim || j.y + TY >= I.ylim) J.face_in_pml = false;
    return J;
}
} // namespace ffipg
