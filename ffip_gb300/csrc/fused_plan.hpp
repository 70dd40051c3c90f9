// Host side of the fused pass's split of a time step's points: which points
// the pass owns, which the face kernel updates (as a list of boxes), and
// which PEC / PMC faces the pass mirrors into the halo of its first tiles.
// Plain C++ (no CUDA), shared by the CUDA backend and the host tests.
#pragma once
#include <algorithm>
#include <cstdint>
#include <stdexcept>

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
} // namespace ffipg
