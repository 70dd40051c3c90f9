// TEST INFRASTRUCTURE — not part of the shipped library.
//
// Host emulation backend: runs the per-point update rules of
// ffip_gb300/csrc/stencil.cuh (the same functions the CUDA kernels call) in
// plain loops on the CPU, so that the engine's set-up, layout, sequencing and
// output logic can be checked against the oracle without a GPU.  Built by
// tests/emu/build_emu.py into tests/_build/libffip_emu.so, which exports the
// same ffip_* C functions as the product library.  The fused pass is not
// emulated (it is a CUDA-only tiling of the same rules).
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "engine.hpp"

namespace ffipg
{
namespace
{
class HostBackend : public Backend
{
public:
    void *alloc(size_t bytes) override
    {
        void *p = std::calloc(bytes ? bytes : 1, 1);
        if (!p) throw std::bad_alloc();
        return p;
    }
    void release(void *p) override { std::free(p); }
    void h2d(void *d, const void *s, size_t b) override
    {
        h2d_bytes += b;
        std::memcpy(d, s, b);
    }
    void d2h(void *d, const void *s, size_t b) override
    {
        d2h_bytes += b;
        std::memcpy(d, s, b);
    }
    void zero(void *p, size_t b) override { std::memset(p, 0, b); }
    void sync() override {}

    template <typename T>
    void update_t(const SideParams<T> &p, bool is_e)
    {
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < p.Mz; ++k)
            for (int j = 0; j < p.My; ++j)
                for (int i = 0; i < p.Mx; ++i)
                    for (int c = 0; c < 3; ++c)
                    {
                        if (i < p.vlo[c][0] || i > p.vhi[c][0] || j < p.vlo[c][1] || j > p.vhi[c][1] || k < p.vlo[c][2] || k > p.vhi[c][2]) continue;
                        if (is_e)
                        {
                            if (c == 0) update_point<T, 0>(p, i, j, k);
                            else if (c == 1) update_point<T, 1>(p, i, j, k);
                            else update_point<T, 2>(p, i, j, k);
                        }
                        else
                        {
                            if (c == 0) update_point<T, 3>(p, i, j, k);
                            else if (c == 1) update_point<T, 4>(p, i, j, k);
                            else update_point<T, 5>(p, i, j, k);
                        }
                    }
    }
    void update(const SideParams<double> &p, bool e) override { update_t(p, e); }
    void update(const SideParams<float> &p, bool e) override { update_t(p, e); }

    template <typename T>
    void sources_t(const SourceParams<T> &p)
    {
        for (int q = 0; q < p.npts; ++q) source_point<T>(p, q);
    }
    void sources(const SourceParams<double> &p) override { sources_t(p); }
    void sources(const SourceParams<float> &p) override { sources_t(p); }

    template <typename T>
    void ghosts_t(const GhostParams<T> &p)
    {
        for (int f = 0; f < p.nfaces; ++f)
            for (int v = 0; v < p.faces[f].v1; ++v)
                for (int u = 0; u < p.faces[f].u1; ++u) ghost_point<T>(p, f, u, v);
    }
    void ghosts(const GhostParams<double> &p) override { ghosts_t(p); }
    void ghosts(const GhostParams<float> &p) override { ghosts_t(p); }

    template <typename T>
    void probe_t(const T *f, const int64_t *lin, const double *w, int n, double *out)
    {
        double r = 0;
        for (int q = 0; q < n; ++q) r += (double)f[lin[q]] * w[q];
        *out = r;
    }
    void probe(const double *f, const int64_t *l, const double *w, int n, double *o) override { probe_t(f, l, w, n, o); }
    void probe(const float *f, const int64_t *l, const double *w, int n, double *o) override { probe_t(f, l, w, n, o); }
    template <typename T>
    bool any_nonfinite_t(const T *const *f, int nf, int64_t n)
    {
        for (int i = 0; i < nf; ++i)
            for (int64_t t = 0; t < n; ++t)
                if (!std::isfinite(f[i][t])) return true;
        return false;
    }
    bool any_nonfinite(const double *const *f, int nf, int64_t n) override { return any_nonfinite_t(f, nf, n); }
    bool any_nonfinite(const float *const *f, int nf, int64_t n) override { return any_nonfinite_t(f, nf, n); }
    void flux(const FluxArgs &A, double *out) override
    {
        const int64_t np = (int64_t)A.n[0] * A.n[1] * A.n[2];
        for (int f = 0; f < A.nf; ++f)
        {
            double s = 0;
            for (int64_t t = 0; t < np; ++t) s += flux_point(A, t, f);
            out[f] = s;
        }
    }
    void dft_norm(const double *re, const double *im, int64_t n, double *out) override
    {
        double s = 0;
        for (int64_t i = 0; i < n; ++i) s += re[i] * re[i] + im[i] * im[i];
        *out = s;
    }
    const char *name() const override { return "host-emulation"; }
    double timed(const std::function<void()> &f) override
    {
        f();
        return 0.0;
    }
};
} // namespace

Backend *new_default_backend(int) { return new HostBackend(); }
void *backend_stream(Backend *) { return nullptr; }
int adjoint_transpose(const double *, uint64_t, const double *, uint64_t, const double *, uint64_t, const double *, uint64_t,
                      double *)
{
    throw std::runtime_error("not emulated");
}
int adjoint_sensitivity(double, double, double, double, const double *, const double *, const double *, const double *, uint64_t,
                        const double *, uint64_t, const double *, uint64_t, const double *, uint64_t, double *)
{
    throw std::runtime_error("not emulated");
}
int adjoint_transpose_noalloc(const double *, uint64_t, const double *, uint64_t, const double *, uint64_t, const double *,
                              uint64_t, double *)
{
    throw std::runtime_error("not emulated");
}
uint64_t adjoint_transpose_noalloc_capacity() { return uint64_t(1) << 20; }
int to_convolve(const double *, int, int, const double *, int, int, double *, int)
{
    throw std::runtime_error("not emulated");
}
int check_inside(const double *, uint64_t, const double *, uint64_t, unsigned char *)
{
    throw std::runtime_error("not emulated");
}
int sg_gemm(int, int, int, const void *, int64_t, int64_t, const void *, int64_t, int64_t, float *, int64_t, int64_t,
            const float *, int, void *, int)
{
    throw std::runtime_error("not emulated");
}
int sg_check() { throw std::runtime_error("not emulated"); }
int sg_im2col_t(const void *, const int *, const int *, const int *, const int *, void *, void *)
{
    throw std::runtime_error("not emulated");
}
int sg_im2col(const void *, const int *, const int *, const int *, const int *, void *, void *)
{
    throw std::runtime_error("not emulated");
}
int sg_col2im(const float *, const int *, const int *, const int *, const int *, float *, void *)
{
    throw std::runtime_error("not emulated");
}
} // namespace ffipg

// ---------------------------------------------------------------------------
// Test hook: the host half of the fused pass's split of a step's points
// (ffip_gb300/csrc/fused_plan.hpp, the code the CUDA backend runs before each
// pass) checked on a config's plan without a GPU.  Tile shape of the CPML
// instance (which sets xlim / ylim): 32 x 8.
#include <string>
#include <vector>

#include "fused_plan.hpp"

extern "C" int ffip_emu_fused_partition_check(const char *config_json, char *msg, uint64_t msg_len)
{
    using namespace ffipg;
    auto fail = [&](const std::string &m) {
        if (msg && msg_len) std::snprintf(msg, msg_len, "%s", m.c_str());
        return 1;
    };
    try
    {
        Json cfg = Json::parse(config_json);
        Plan P;
        build_plan(cfg, {}, P);
        GhostFace all[kMaxFaces];
        const int nf = build_ghost_faces(P, all, kMaxFaces);
        std::vector<GhostFace> hf;
        for (int f = 0; f < nf; ++f)
            if (all[f].comp >= 3) hf.push_back(all[f]);
        int vlo[2][3][3], vhi[2][3][3];
        int xend = 0, yend = 0;
        for (int c = 0; c < 6; ++c)
            for (int a = 0; a < 3; ++a)
            {
                vlo[c / 3][c % 3][a] = P.vlo[c][a];
                vhi[c / 3][c % 3][a] = P.vhi[c][a];
                if (a == 0) xend = std::max(xend, P.vhi[c][0] + 1);
                if (a == 1) yend = std::max(yend, P.vhi[c][1] + 1);
            }
        int nbx, nby, xlim, ylim;
        fused_limits(xend, yend, kXFirst, 32, 8, nbx, nby, xlim, ylim);
        const FusedOwnership own = fused_ownership(vlo[0], vhi[0], hf.data(), (int)hf.size(), kXFirst, true);
        const FaceList fl[2] = {fused_face_list(vlo[0], vhi[0], own.elo, own.ehi, xlim, ylim),
                                fused_face_list(vlo[1], vhi[1], nullptr, nullptr, xlim, ylim)};
        auto owned = [&](int side, int c, int i, int j, int k) {
            if (i >= xlim || j >= ylim) return false;
            const int(*lo)[3] = side == 0 ? own.elo : vlo[1];
            const int(*hi)[3] = side == 0 ? own.ehi : vhi[1];
            return i >= lo[c][0] && i <= hi[c][0] && j >= lo[c][1] && j <= hi[c][1] && k >= lo[c][2] && k <= hi[c][2];
        };
        auto in_box = [&](const FaceList &B, int c, int i, int j, int k) {
            int hits = 0;
            for (int b = 0; b < B.n; ++b)
            {
                const FaceBox &X = B.b[b];
                const int64_t end = b + 1 < B.n ? B.b[b + 1].start : B.total;
                const int nk = (int)((end - X.start) / ((int64_t)X.ni * X.nj));
                hits += X.comp == c && i >= X.i0 && i < X.i0 + X.ni && j >= X.j0 && j < X.j0 + X.nj && k >= X.k0 && k < X.k0 + nk;
            }
            return hits;
        };
        // a ghost position of H component h: on a face's ghost plane, inside its in-plane range
        auto ghost_of = [&](int h, const int q[3]) -> const GhostFace * {
            for (const GhostFace &G : hf)
            {
                if (G.comp != 3 + h || q[G.axis] != G.dst) continue;
                int au, av;
                ghost_axes(G.axis, au, av);
                if (q[au] >= G.u0 && q[au] < G.u0 + G.u1 && q[av] >= G.v0 && q[av] < G.v0 + G.v1) return &G;
            }
            return nullptr;
        };
        for (int side = 0; side < 2; ++side)
            for (int c = 0; c < 3; ++c)
                for (int k = vlo[side][c][2]; k <= vhi[side][c][2]; ++k)
                    for (int j = vlo[side][c][1]; j <= vhi[side][c][1]; ++j)
                        for (int i = vlo[side][c][0]; i <= vhi[side][c][0]; ++i)
                        {
                            const bool o = owned(side, c, i, j, k);
                            const int f = in_box(fl[side], c, i, j, k);
                            if ((o ? 1 : 0) + f != 1)
                                return fail("point " + std::to_string(side * 3 + c) + " (" + std::to_string(i) + "," +
                                            std::to_string(j) + "," + std::to_string(k) + "): owned " + std::to_string(o) +
                                            ", face boxes " + std::to_string(f));
                            if (side != 0 || !o) continue;
                            // the H values the pass's E update reads
                            const int pairs[2][2] = {{(c + 2) % 3, (c + 1) % 3}, {(c + 1) % 3, (c + 2) % 3}};
                            for (const auto &hp : pairs)
                                for (int d = 0; d <= 1; ++d)
                                {
                                    int q[3] = {i, j, k};
                                    q[hp[1]] -= d;
                                    const GhostFace *G = ghost_of(hp[0], q);
                                    if (!G) continue;
                                    const int first[2] = {kXFirst, 1};
                                    const bool mirrored = G->axis < 2 && own.hmirror[G->axis] == G->mult && own.hghost[G->axis] == G->dst &&
                                                          q[G->axis] == first[G->axis] - 1 && G->src == G->dst + 1;
                                    if (!mirrored)
                                        return fail("owned E point " + std::to_string(c) + " (" + std::to_string(i) + "," +
                                                    std::to_string(j) + "," + std::to_string(k) + ") reads the H ghost of face axis " +
                                                    std::to_string(G->axis));
                                }
                        }
        if (msg && msg_len) std::snprintf(msg, msg_len, "ok %d H faces, %d + %d face boxes, mirror %d %d", (int)hf.size(), fl[0].n,
                                          fl[1].n, own.hmirror[0], own.hmirror[1]);
        return 0;
    }
    catch (const std::exception &e)
    {
        return fail(std::string("error: ") + e.what());
    }
}

// Test hook: the fused pass's CTA job lists (fused_plan.hpp fused_jobs, which
// the CUDA backend runs once per grid) built from a config's plan, with the
// interior instance's tile width tx (64: fp32, 32: fp64) and z chunks of at
// most kch planes, checked: every 32-column unit below xlim, 8-row tile and
// valid z plane belongs to exactly one job; no job of the instance without
// CPML code meets CPML in its tile, low-x / low-y halo or planes (or the plane
// below its first); jobs start on unit and tile boundaries inside the valid
// z range.
extern "C" int ffip_emu_fused_jobs_check(const char *config_json, int tx, int kch, char *msg, uint64_t msg_len)
{
    using namespace ffipg;
    auto fail = [&](const std::string &m) {
        if (msg && msg_len) std::snprintf(msg, msg_len, "%s", m.c_str());
        return 1;
    };
    try
    {
        Json cfg = Json::parse(config_json);
        Plan P;
        build_plan(cfg, {}, P);
        if (P.rasterize != "host") rasterize_media(P);
        const int TXP = 32, TY = 8;
        int xend = 0, yend = 0, kbeg = P.M[2], kend = 0;
        for (int c = 0; c < 6; ++c)
        {
            xend = std::max(xend, P.vhi[c][0] + 1);
            yend = std::max(yend, P.vhi[c][1] + 1);
            kbeg = std::min(kbeg, P.vlo[c][2]);
            kend = std::max(kend, P.vhi[c][2] + 1);
        }
        kend = std::max(kend, kbeg + 1);
        JobInputs I;
        fused_limits(xend, yend, kXFirst, TXP, TY, I.nbx, I.nby, I.xlim, I.ylim);
        const int len[3] = {xend, P.M[1], P.M[2]};
        for (int a = 0; a < 3; ++a)
        {
            I.pml[a].assign(len[a], 0);
            for (int q = 0; q < 2; ++q)
                for (int i = 0; i < len[a] && i < (int)P.pml_c[a][q].size(); ++i) I.pml[a][i] |= P.pml_c[a][q][i] != 0;
        }
        I.My = P.M[1];
        I.Mz = P.M[2];
        for (int c = 0; c < 3; ++c)
        {
            const SlotList &S = P.slots[c];
            if (S.lin.empty()) continue;
            I.rows[c].assign((size_t)I.My * I.Mz, RowRange{1, 0});
            for (int64_t l : S.lin)
            {
                const int i = (int)(l % P.Mx_pad), j = (int)((l / P.Mx_pad) % P.M[1]), k = (int)(l / P.plane());
                RowRange &r = I.rows[c][(size_t)k * I.My + j];
                if (r.lo > r.hi) r.lo = r.hi = i;
                else
                {
                    r.lo = std::min(r.lo, i);
                    r.hi = std::max(r.hi, i);
                }
            }
        }
        for (const DftUnit &U : P.units)
            if (U.has_local)
            {
                DftBox d;
                for (int a = 0; a < 3; ++a)
                {
                    d.i0[a] = U.i0[a];
                    d.ld[a] = U.ldim[a];
                }
                d.nf = (int)U.freqs.size();
                I.dft.push_back(d);
            }
        I.kbeg = kbeg;
        I.kend = kend;
        I.TX = tx;
        I.TXP = TXP;
        I.TY = TY;
        I.KCH = kch;
        const JobLists J = fused_jobs(I, kXFirst, false, 4, true, false);
        auto anyp = [&](int a, int lo, int hi) {
            for (int i = std::max(lo, 0); i <= std::min(hi, len[a] - 1); ++i)
                if (I.pml[a][i]) return true;
            return false;
        };
        const int nu = std::max(I.nbx, 1), nby = std::max(I.nby, 1), nz = kend - kbeg;
        std::vector<int> cover((size_t)nu * nby * nz, 0);
        auto mark = [&](const JobBox &j, int width) -> std::string {
            if ((j.x - kXFirst) % TXP != 0 || (j.y - 1) % TY != 0 || j.z < kbeg || j.w > kend || j.z >= j.w)
                return "a job off the unit / tile grid or the z range";
            for (int x0 = j.x; x0 < j.x + width; x0 += TXP)
            {
                const int u = (x0 - kXFirst) / TXP, by = (j.y - 1) / TY;
                if (u >= nu || by >= nby) return "a job beyond the units / tiles";
                for (int z = j.z; z < j.w; ++z) ++cover[((size_t)by * nu + u) * nz + (z - kbeg)];
            }
            return "";
        };
        for (const JobBox &j : J.b)
        {
            const std::string e = mark(j, TXP);
            if (!e.empty()) return fail(e);
            if (j.x >= I.xlim) return fail("a CPML job at or beyond xlim");
        }
        for (const JobBox &j : J.in)
        {
            const std::string e = mark(j, tx);
            if (!e.empty()) return fail(e);
            if (anyp(0, j.x - 1, j.x + tx - 1) || anyp(1, j.y - 1, j.y + TY - 1) || anyp(2, j.z - 1, j.w - 1))
                return fail("an interior job at (" + std::to_string(j.x) + "," + std::to_string(j.y) + "," + std::to_string(j.z) +
                            ") meets CPML");
        }
        for (int by = 0; by < nby; ++by)
            for (int u = 0; u < nu; ++u)
                for (int z = 0; z < nz; ++z)
                {
                    const int n = cover[((size_t)by * nu + u) * nz + z];
                    const bool below = kXFirst + u * TXP < I.xlim;
                    if ((below && n != 1) || n > 1)
                        return fail("unit " + std::to_string(u) + ", tile " + std::to_string(by) + ", plane " +
                                    std::to_string(z + kbeg) + " covered " + std::to_string(n) + " times");
                }
        if (msg && msg_len)
            std::snprintf(msg, msg_len, "ok %d CPML jobs, %d interior jobs, %d units x %d tiles x %d planes", (int)J.b.size(),
                          (int)J.in.size(), nu, nby, nz);
        return 0;
    }
    catch (const std::exception &e)
    {
        return fail(std::string("error: ") + e.what());
    }
}
