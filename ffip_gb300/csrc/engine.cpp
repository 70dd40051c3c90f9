// Engine<T>: device state + half-step sequencing.  Backend-agnostic host code.
#include "engine.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>

namespace ffipg
{
namespace
{
template <typename T>
struct DevSlots
{
    int *map{nullptr};
    RowRange *rows{nullptr};
    T *g{nullptr}, *coef{nullptr}, *inv{nullptr};
    uint8_t *group{nullptr};
    SlotRec<T> *rec{nullptr};
    T *A{nullptr}, *amp{nullptr}, *P{nullptr}, *P1{nullptr};
    T *Pb{nullptr}, *P1b{nullptr};  // fused pass, H side: the other P / J buffers (ping-pong between steps)
    int64_t n{0};
    int stride{0};
    bool poles{false};
};

struct DevSources
{
    int npts{0};
    uint8_t *comp{nullptr};
    int64_t *lin{nullptr};
    int *off{nullptr};
    double *amp{nullptr}, *start{nullptr}, *end{nullptr}, *width{nullptr};
    uint8_t *kind{nullptr};
    int *moff{nullptr}, *munit{nullptr};
    int64_t *mlin{nullptr};
    double max_end{0};
};

template <typename T>
class Engine : public EngineBase
{
public:
    Engine(Plan &&plan, Backend *be) : P_(std::move(plan)), be_(be) { init(); }
    ~Engine() override { free_all(); }

    const Plan &plan() const override { return P_; }
    bool fused() const override { return fused_; }
    int64_t time_step() const override { return ts_; }
    int64_t launches() const override { return nlaunch_; }

    void step(int64_t n) override
    {
        for (int64_t s = 0; s < n; ++s) one_step();
    }

    void run(const Json &stop) override;
    std::vector<OutputGroup> outputs() override;
    void reset() override;
    void set_density(const std::string &dataset, const double *rho, uint64_t n) override;
    void set_source_data(const std::map<std::string, std::vector<double>> &data) override;
    double bytes_per_step() const override { return bytes_per_step_; }
    double pass_bytes_per_step() const override { return pass_bytes_per_step_; }
    void media_checksum(uint64_t out[6]) override;
    bool device_media() const override { return device_media_; }
    std::vector<double> flux(const std::string &e1_group, const std::string &h2_group, const std::vector<double> &x,
                             const std::vector<double> &y, const std::vector<double> &z, const std::vector<double> &w,
                             const std::vector<double> &freqs) override;

private:
    Plan P_;
    Backend *be_;
    std::vector<void *> allocs_;       // freed with the engine
    std::vector<void *> slot_allocs_;  // freed when the media change
    std::vector<void *> src_allocs_;   // freed when the sources change
    T *buf_[2][6]{};                   // field buffers; [1] only with the fused pass
    int cur_{0};
    T *psi_[6][2]{};
    T *psih_b_[3][2]{};                // second H psi buffer for the fused pass
    T *pml_b_[3][2]{}, *pml_c_[3][2]{}, *pml_ik_[3][2]{};
    DevSlots<T> slots_[6];
    uint8_t *grp_np_[2]{}, *grp_pool_[2]{};
    T *pool_c_[2]{};
    DevSources src_[2];
    std::vector<double *> dre_, dim_;
    std::vector<int> side_units_[2];
    SideParams<T> sp_[2];
    SourceParams<T> srcp_[2];
    GhostParams<T> gp_{};
    GhostParams<T> gph_{};  // the H faces of gp_ (the fused pass fills them between its halves)
    GhostParams<T> gpe_{};  // the E faces of gp_ (all that is left to fill after a fused step)
    bool fused_{false};
    int64_t ts_{0};
    int64_t nlaunch_{0};
    double *scratch_{nullptr};
    int64_t scratch_n_{0};
    double bytes_per_step_{0};
    double pass_bytes_per_step_{0};
    bool device_media_{false};   // media rasterised by the backend
    int64_t pole_sum_[6]{};      // active poles summed over each component's slots
    bool comp_poles_[6]{};       // a component has slots with poles

    // allocation lifetimes: with the engine, until the media change, until
    // the sources change
    enum Life { kEngine = 0, kMedia = 1, kSources = 2 };
    template <typename U>
    U *dalloc(size_t n, int life = kEngine)
    {
        if (n == 0) return nullptr;
        void *p = be_->alloc(n * sizeof(U));
        (life == kMedia ? slot_allocs_ : life == kSources ? src_allocs_ : allocs_).push_back(p);
        return (U *)p;
    }
    template <typename U>
    U *upload(const std::vector<U> &v, int life = kEngine)
    {
        U *p = dalloc<U>(v.size(), life);
        if (p) be_->h2d(p, v.data(), v.size() * sizeof(U));
        return p;
    }
    void free_all()
    {
        for (void *p : slot_allocs_) be_->release(p);
        for (void *p : src_allocs_) be_->release(p);
        for (void *p : allocs_) be_->release(p);
        slot_allocs_.clear();
        src_allocs_.clear();
        allocs_.clear();
    }

    void init();
    void media();
    void init_media();
    void init_media_device();
    void upload_pole_tables();
    void init_sources();
    void init_dft();
    void init_ghosts();
    void alloc_fused_pole_state();
    void bind_params();
    void compute_bytes();
    void set_phases(int side, double t, double (*phase)[2]);
    void one_step();
    void check_finite();
    void ensure_scratch(int64_t n)
    {
        if (n <= scratch_n_) return;
        if (scratch_) be_->release(scratch_);
        scratch_n_ = std::max<int64_t>(n, 1024);
        scratch_ = (double *)be_->alloc(scratch_n_ * sizeof(double));
    }
};

template <typename T>
void Engine<T>::init()
{
    const int64_t cells = P_.cells();
    // CPML tables
    bool pml = P_.any_pml;
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 2; ++q)
        {
            if (!pml) continue;
            std::vector<T> b(P_.M[a]), c(P_.M[a]), ik(P_.M[a]);
            for (int i = 0; i < P_.M[a]; ++i)
            {
                b[i] = (T)P_.pml_b[a][q][i];
                c[i] = (T)P_.pml_c[a][q][i];
                ik[i] = (T)(1 / P_.pml_k[a][q][i]);
            }
            pml_b_[a][q] = upload(b);
            pml_c_[a][q] = upload(c);
            pml_ik_[a][q] = upload(ik);
        }
    // the media: slot tables on the device (rasterised there, or uploaded
    // from the host's rasterisation)
    media();
    // fused pass eligibility (a CUDA backend)
    const bool eligible = be_->has_fused();
    if (P_.engine == "fused" && !eligible) throw std::runtime_error("engine \"fused\" requested but the backend has no fused pass");
    if (P_.engine != "auto" && P_.engine != "fused" && P_.engine != "unfused")
        throw std::runtime_error("engine must be \"auto\", \"fused\" or \"unfused\"");
    fused_ = eligible && P_.engine != "unfused";
    alloc_fused_pole_state();
    for (int c = 0; c < 6; ++c)
    {
        buf_[0][c] = dalloc<T>(cells);
        if (fused_) buf_[1][c] = dalloc<T>(cells);
    }
    for (int c = 0; c < 6; ++c)
        for (int s = 0; s < 2; ++s)
        {
            int a = (c % 3 + 1 + s) % 3;
            int q = comp_parity(c, a);
            bool need = false;
            if (pml)
                for (double v : P_.pml_c[a][q]) need = need || v != 0;
            if (need)
            {
                psi_[c][s] = dalloc<T>(cells);
                if (fused_ && c >= 3) psih_b_[c - 3][s] = dalloc<T>(cells);
            }
        }
    init_dft();
    init_sources();
    init_ghosts();
    bind_params();
    compute_bytes();
}

template <typename T>
void Engine<T>::media()
{
    if (P_.rasterize == "device" && !be_->can_rasterize()) throw std::runtime_error("rasterize \"device\": the backend cannot");
    if (P_.rasterize == "device" || (P_.rasterize == "auto" && be_->can_rasterize()))
    {
        try
        {
            init_media_device();
            return;
        }
        catch (const RasterUnsupported &)
        {
            // a geometry the device rasterisation does not cover ("auto"
            // falls back to the host)
            if (P_.rasterize == "device") throw;
        }
    }
    if (P_.rasterize != "host") rasterize_media(P_);
    init_media();
}

template <typename T>
void Engine<T>::init_media_device()
{
    for (void *p : slot_allocs_) be_->release(p);
    slot_allocs_.clear();
    for (int side = 0; side < 2; ++side)
    {
        P_.groups[side].clear();
        P_.group_index[side].clear();
    }
    for (int c = 0; c < 6; ++c) P_.slots[c] = SlotList();
    RasterComp out[6];
    std::vector<PoleGroup> groups[2];
    be_->rasterize(P_, sizeof(T) == 4, [this](size_t bytes) { return (void *)dalloc<uint8_t>(bytes, kMedia); }, out, groups);
    for (int side = 0; side < 2; ++side)
    {
        P_.groups[side] = groups[side];
        for (size_t g = 0; g < groups[side].size(); ++g) P_.group_index[side][groups[side][g].pool] = (int)g;
    }
    for (int c = 0; c < 6; ++c)
    {
        const RasterComp &R = out[c];
        DevSlots<T> &D = slots_[c];
        D = DevSlots<T>();
        D.n = R.n;
        D.stride = R.stride;
        D.poles = R.stride > 0;
        pole_sum_[c] = R.pole_sum;
        comp_poles_[c] = D.poles;
        if (!D.n) continue;
        D.map = R.map;
        D.rows = R.rows;
        D.g = (T *)R.g;
        D.coef = (T *)R.coef;
        D.inv = (T *)R.inv;
        D.group = R.group;
        D.rec = (SlotRec<T> *)R.rec;
        if (D.poles)
        {
            if (c >= 3) D.A = dalloc<T>(D.n, kMedia);  // H sources are applied before the H update
            D.amp = (T *)R.amp;
            D.P = dalloc<T>((size_t)D.stride * D.n, kMedia);
            D.P1 = dalloc<T>((size_t)D.stride * D.n, kMedia);
        }
    }
    upload_pole_tables();
    device_media_ = true;
}

template <typename T>
void Engine<T>::media_checksum(uint64_t out[6])
{
    // FNV-1a over the tables' bytes, copied back from the device
    auto fnv = [](uint64_t h, const void *p, size_t n) {
        const unsigned char *b = (const unsigned char *)p;
        for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
        return h;
    };
    be_->sync();
    for (int c = 0; c < 6; ++c)
    {
        const DevSlots<T> &D = slots_[c];
        uint64_t h = 1469598103934665603ull;
        h = fnv(h, &D.n, sizeof D.n);
        h = fnv(h, &D.stride, sizeof D.stride);
        auto add = [&](const void *dev, size_t bytes) {
            if (!dev || !bytes) return;
            std::vector<unsigned char> buf(bytes);
            be_->d2h(buf.data(), dev, bytes);
            h = fnv(h, buf.data(), bytes);
        };
        if (D.n)
        {
            add(D.map, (size_t)P_.cells() * sizeof(int));
            add(D.rows, (size_t)P_.M[1] * P_.M[2] * sizeof(RowRange));
            add(D.g, D.n * sizeof(T));
            add(D.coef, D.n * sizeof(T));
            add(D.inv, D.n * sizeof(T));
            add(D.group, D.n);
            add(D.rec, D.n * sizeof(SlotRec<T>));
            add(D.amp, (size_t)D.stride * D.n * sizeof(T));
        }
        out[c] = h;
    }
}

template <typename T>
std::vector<double> Engine<T>::flux(const std::string &e1_group, const std::string &h2_group, const std::vector<double> &x,
                                    const std::vector<double> &y, const std::vector<double> &z, const std::vector<double> &w,
                                    const std::vector<double> &freqs)
{
    if (freqs.empty()) return {};
    if ((int)freqs.size() > kMaxFluxFreqs)
        throw std::runtime_error("flux: at most " + std::to_string(kMaxFluxFreqs) + " frequencies per call");
    if (x.empty() || y.empty() || z.empty() || w.size() != x.size() * y.size() * z.size())
        throw std::runtime_error("flux: the weights must cover the x * y * z integration points");
    // the output grid of a monitor group (the closure's points, dx/2 apart
    // on the doubled grid) as the reference's interpolant sees it
    auto grid = [&](const std::string &group, FluxGrid &G) {
        const DftRequest *req = nullptr;
        for (auto &r : P_.requests)
            if (r.group == group) req = &r;
        if (!req) throw std::runtime_error("flux: no monitor group '" + group + "'");
        const DftUnit &U = P_.units[req->unit];
        G = FluxGrid();
        G.re = dre_[req->unit];
        G.im = dim_[req->unit];
        G.npts = U.npoints();
        for (int a = 0; a < 3; ++a)
        {
            G.ld[a] = U.has_local ? U.ldim[a] : 0;
            G.off[a] = U.has_local ? (U.l1[a] - U.c1[a]) / 2 : 0;
            G.dim[a] = U.dim[a];
            const double s0 = U.c1[a] * (P_.dx / 2), s1 = U.c2[a] * (P_.dx / 2);
            if (U.dim[a] <= 1)
            {
                // one point: widened to +-dx/2, the value repeated
                G.wide[a] = 1;
                G.n[a] = 2;
                G.g0[a] = s0 - P_.dx / 2;
                G.gs[a] = P_.dx;
            }
            else
            {
                G.n[a] = U.dim[a];
                G.g0[a] = s0;
                G.gs[a] = (s1 - s0) / (U.dim[a] - 1);
            }
        }
        for (size_t f = 0; f < freqs.size(); ++f)
        {
            auto it = std::lower_bound(U.freqs.begin(), U.freqs.end(), freqs[f]);
            if (it == U.freqs.end() || *it != freqs[f]) throw std::runtime_error("flux: frequency not registered in '" + group + "'");
            G.fidx[f] = (int)(it - U.freqs.begin());
        }
    };
    FluxArgs A;
    grid(e1_group, A.e1);
    grid(h2_group, A.h2);
    A.nf = (int)freqs.size();
    A.n[0] = (int)x.size();
    A.n[1] = (int)y.size();
    A.n[2] = (int)z.size();
    A.x = x.data();
    A.y = y.data();
    A.z = z.data();
    A.w = w.data();
    std::vector<double> out(freqs.size(), 0.0);
    be_->flux(A, out.data());
    ++nlaunch_;
    return out;
}

template <typename T>
void Engine<T>::init_media()
{
    for (void *p : slot_allocs_) be_->release(p);
    slot_allocs_.clear();
    const int64_t cells = P_.cells();
    for (int c = 0; c < 6; ++c)
    {
        const SlotList &L = P_.slots[c];
        DevSlots<T> &D = slots_[c];
        D = DevSlots<T>();
        D.n = (int64_t)L.lin.size();
        D.stride = L.npole_stride;
        D.poles = L.any_poles;
        if (!D.n) continue;
        if (D.n > std::numeric_limits<int>::max()) throw std::runtime_error("too many material slots for one component");
        std::vector<int> map(cells, -1);
        std::vector<RowRange> rows((size_t)P_.M[1] * P_.M[2], RowRange{1, 0});
        std::vector<T> g(D.n), coef(D.n), inv(D.n);
        std::vector<uint8_t> grp(D.n);
        for (int64_t s = 0; s < D.n; ++s)
        {
            int64_t l = L.lin[s];
            map[l] = (int)s;
            int i = (int)(l % P_.Mx_pad);
            int64_t row = l / P_.Mx_pad;
            RowRange &r = rows[row];
            if (r.lo > r.hi) r.lo = r.hi = i;
            else { r.lo = std::min(r.lo, i); r.hi = std::max(r.hi, i); }
            g[s] = (T)L.g[s];
            coef[s] = (T)(P_.dt / L.g[s]);
            inv[s] = (T)(1 / L.g[s]);
            if (L.group[s] > 255) throw std::runtime_error("more than 256 distinct pole patterns");
            grp[s] = (uint8_t)L.group[s];
        }
        D.map = upload(map, kMedia);
        D.rows = upload(rows, kMedia);
        D.g = upload(g, kMedia);
        D.coef = upload(coef, kMedia);
        D.inv = upload(inv, kMedia);
        D.group = upload(grp, kMedia);
        {
            std::vector<SlotRec<T>> rec(D.n);
            const auto &G = P_.groups[c / 3];
            for (int64_t s = 0; s < D.n; ++s)
            {
                const int np = L.group[s] < (int)G.size() ? (int)G[L.group[s]].pool.size() : 0;
                rec[s] = SlotRec<T>{coef[s], inv[s], g[s], (T)(grp[s] + 256 * np)};
            }
            D.rec = upload(rec, kMedia);
        }
        if (D.poles)
        {
            if (c >= 3) D.A = dalloc<T>(D.n, kMedia);  // H sources are applied before the H update
            std::vector<T> amp(L.amp.size());
            for (size_t q = 0; q < amp.size(); ++q) amp[q] = (T)L.amp[q];
            D.amp = upload(amp, kMedia);
            D.P = dalloc<T>(amp.size(), kMedia);
            D.P1 = dalloc<T>(amp.size(), kMedia);
        }
    }
    for (int c = 0; c < 6; ++c)
    {
        const SlotList &L = P_.slots[c];
        int64_t ps = 0;
        for (size_t q = 0; q < L.group.size(); ++q) ps += (int64_t)P_.groups[c / 3][L.group[q]].pool.size();
        pole_sum_[c] = ps;
        comp_poles_[c] = L.any_poles;
    }
    upload_pole_tables();
    device_media_ = false;
}

template <typename T>
void Engine<T>::upload_pole_tables()
{
    for (int side = 0; side < 2; ++side)
    {
        const auto &G = P_.groups[side];
        std::vector<uint8_t> np(std::max<size_t>(G.size(), 1), 0), pool(std::max<size_t>(G.size(), 1) * kMaxPolesDev, 0);
        for (size_t g = 0; g < G.size(); ++g)
        {
            np[g] = (uint8_t)G[g].pool.size();
            for (size_t q = 0; q < G[g].pool.size(); ++q)
            {
                if (G[g].pool[q] > 255) throw std::runtime_error("susceptibility pool larger than 256");
                pool[g * kMaxPolesDev + q] = (uint8_t)G[g].pool[q];
            }
        }
        grp_np_[side] = upload(np, kMedia);
        grp_pool_[side] = upload(pool, kMedia);
        std::vector<T> pc(std::max<size_t>(P_.pool_coef[side].size(), 1) * 3, T(0));
        for (size_t q = 0; q < P_.pool_coef[side].size(); ++q)
            for (int t = 0; t < 3; ++t) pc[3 * q + t] = (T)P_.pool_coef[side][q][t];
        pool_c_[side] = upload(pc, kMedia);
    }
}

template <typename T>
void Engine<T>::init_dft()
{
    dre_.assign(P_.units.size(), nullptr);
    dim_.assign(P_.units.size(), nullptr);
    side_units_[0].clear();
    side_units_[1].clear();
    int nphase[2] = {0, 0};
    for (size_t u = 0; u < P_.units.size(); ++u)
    {
        const DftUnit &U = P_.units[u];
        int side = U.comp < 3 ? 0 : 1;
        int64_t n = U.npoints() * (int64_t)U.freqs.size();
        dre_[u] = dalloc<double>(n);
        dim_[u] = dalloc<double>(n);
        if (!U.has_local) continue;
        side_units_[side].push_back((int)u);
        nphase[side] += (int)U.freqs.size();
    }
    for (int side = 0; side < 2; ++side)
    {
        if ((int)side_units_[side].size() > kMaxUnitsPerSide)
            throw std::runtime_error("too many DFT monitors on one side (limit " + std::to_string(kMaxUnitsPerSide) + ")");
        if (nphase[side] > kMaxPhases)
            throw std::runtime_error("too many (monitor, frequency) pairs on one side (limit " + std::to_string(kMaxPhases) + ")");
    }
}

template <typename T>
void Engine<T>::init_sources()
{
    for (int side = 0; side < 2; ++side)
    {
        DevSources &S = src_[side];
        S = DevSources();
        const auto &dl = P_.dipoles[side];
        if (dl.empty()) continue;
        std::map<std::pair<int, int64_t>, int> pid;
        std::vector<std::vector<int>> members;
        std::vector<int> comp;
        std::vector<int64_t> lin;
        for (size_t d = 0; d < dl.size(); ++d)
        {
            auto key = std::make_pair(dl[d].comp, dl[d].lin);
            auto it = pid.find(key);
            int id;
            if (it == pid.end())
            {
                id = (int)members.size();
                pid[key] = id;
                members.emplace_back();
                comp.push_back(dl[d].comp);
                lin.push_back(dl[d].lin);
            }
            else
                id = it->second;
            members[id].push_back((int)d);
            S.max_end = std::max(S.max_end, dl[d].end);
        }
        S.npts = (int)members.size();
        std::vector<uint8_t> c8(S.npts), kind;
        std::vector<int> off(1, 0);
        std::vector<double> amp, st, en, wd;
        for (int q = 0; q < S.npts; ++q)
        {
            c8[q] = (uint8_t)(comp[q] - 3 * side);
            for (int d : members[q])
            {
                amp.push_back(dl[d].amp);
                st.push_back(dl[d].start);
                en.push_back(dl[d].end);
                wd.push_back(dl[d].width);
                kind.push_back((uint8_t)dl[d].kind);
            }
            off.push_back((int)amp.size());
        }
        S.comp = upload(c8, kSources);
        S.lin = upload(lin, kSources);
        S.off = upload(off, kSources);
        S.amp = upload(amp, kSources);
        S.start = upload(st, kSources);
        S.end = upload(en, kSources);
        S.width = upload(wd, kSources);
        S.kind = upload(kind, kSources);
        // DFT memberships of each source point (applied with the E sources,
        // which are added after the fused/unfused E update)
        std::vector<int> moff(1, 0), munit;
        std::vector<int64_t> mlin;
        for (int q = 0; q < S.npts; ++q)
        {
            int64_t l = lin[q];
            int i = (int)(l % P_.Mx_pad), j = (int)((l / P_.Mx_pad) % P_.M[1]), k = (int)(l / P_.plane());
            for (size_t su = 0; su < side_units_[side].size(); ++su)
            {
                const DftUnit &U = P_.units[side_units_[side][su]];
                if (U.comp != comp[q]) continue;
                int li = i - U.i0[0], lj = j - U.i0[1], lk = k - U.i0[2];
                if (li < 0 || lj < 0 || lk < 0 || li >= U.ldim[0] || lj >= U.ldim[1] || lk >= U.ldim[2]) continue;
                munit.push_back((int)su);
                mlin.push_back(((int64_t)lk * U.ldim[1] + lj) * U.ldim[0] + li);
            }
            moff.push_back((int)munit.size());
        }
        S.moff = upload(moff, kSources);
        S.munit = upload(munit, kSources);
        S.mlin = upload(mlin, kSources);
    }
}

// The fused pass keeps the H side's pole state in two buffers (neighbouring
// tiles recompute halo H from the old state while the owner writes the new),
// allocated with the media
template <typename T>
void Engine<T>::alloc_fused_pole_state()
{
    if (!fused_) return;
    for (int c = 3; c < 6; ++c)
    {
        DevSlots<T> &D = slots_[c];
        if (!D.P) continue;
        D.Pb = dalloc<T>((size_t)D.stride * D.n, kMedia);
        D.P1b = dalloc<T>((size_t)D.stride * D.n, kMedia);
    }
}

} // namespace

int build_ghost_faces(const Plan &P, GhostFace *faces, int max_faces)
{
    // Faces filled after every half step, src/fields.cpp:327-482:
    //   PEC/PMC: ghost(lo-1) = mult * value(lo+1), mult = (lo odd ? phase : -phase)
    //   periodic: ghost(lo-1) = value(hi-1), ghost(hi+1) = value(lo+1)
    int nf = 0;
    for (int a = 0; a < 3; ++a)
        for (int side = 0; side < 2; ++side)
        {
            int bc = P.bc[a][side];
            if (bc == BC_NONE || bc == BC_SYNC) continue;
            int edge = side == 0 ? P.lo[a] : P.hi[a];
            int ghost = side == 0 ? P.lo[a] - 1 : P.hi[a] + 1;
            int src;
            int mult = 1;
            if (bc == BC_PERIOD) src = side == 0 ? P.hi[a] - 1 : P.lo[a] + 1;
            else
            {
                src = side == 0 ? P.lo[a] + 1 : P.hi[a] - 1;
                int phase = bc == BC_PEC ? -1 : 1;
                mult = (edge & 1) ? phase : -phase;
            }
            for (int c = 0; c < 6; ++c)
            {
                if (comp_parity(c, a) != (ghost & 1)) continue;
                if (nf >= max_faces) throw std::runtime_error("too many ghost faces");
                GhostFace &F = faces[nf++];
                F.comp = c;
                F.axis = a;
                F.src = P.index_of(a, src);
                F.dst = P.index_of(a, ghost);
                F.mult = mult;
                int au, av;
                ghost_axes(a, au, av);
                F.u0 = P.vlo[c][au];
                F.u1 = std::max(0, P.vhi[c][au] - P.vlo[c][au] + 1);
                F.v0 = P.vlo[c][av];
                F.v1 = std::max(0, P.vhi[c][av] - P.vlo[c][av] + 1);
            }
        }
    return nf;
}

namespace
{
template <typename T>
void Engine<T>::init_ghosts()
{
    gp_ = GhostParams<T>();
    const int nf = build_ghost_faces(P_, gp_.faces, kMaxFaces);
    gp_.nfaces = nf;
    gp_.sy = P_.Mx_pad;
    gp_.sz = P_.plane();
    gph_ = GhostParams<T>();
    gph_.sy = gp_.sy;
    gph_.sz = gp_.sz;
    gpe_ = gph_;
    gpe_.nfaces = 0;
    for (int f = 0; f < nf; ++f)
        if (gp_.faces[f].comp >= 3) gph_.faces[gph_.nfaces++] = gp_.faces[f];
        else gpe_.faces[gpe_.nfaces++] = gp_.faces[f];
}

template <typename T>
void Engine<T>::bind_params()
{
    for (int side = 0; side < 2; ++side)
    {
        SideParams<T> &p = sp_[side];
        p = SideParams<T>();
        p.Mx = P_.Mx_pad;
        p.My = P_.M[1];
        p.Mz = P_.M[2];
        p.sy = P_.Mx_pad;
        p.sz = P_.plane();
        for (int c = 0; c < 3; ++c)
            for (int a = 0; a < 3; ++a)
            {
                p.vlo[c][a] = P_.vlo[3 * side + c][a];
                p.vhi[c][a] = P_.vhi[3 * side + c][a];
                p.par[c][a] = comp_parity(3 * side + c, a);
            }
        p.inv_dx = (T)(1 / P_.dx);
        p.dt = (T)P_.dt;
        for (int c = 0; c < 3; ++c)
        {
            p.f[c] = buf_[cur_][3 * side + c];
            p.o[c] = buf_[cur_][3 * (1 - side) + c];
            p.psi[c][0] = psi_[3 * side + c][0];
            p.psi[c][1] = psi_[3 * side + c][1];
        }
        for (int a = 0; a < 3; ++a)
            for (int q = 0; q < 2; ++q)
            {
                p.pb[a][q] = pml_b_[a][q];
                p.pc[a][q] = pml_c_[a][q];
                p.pik[a][q] = pml_ik_[a][q];
            }
        p.g_def = (T)P_.g_default[side];
        p.coef_def = (T)(P_.dt / P_.g_default[side]);
        for (int c = 0; c < 3; ++c)
        {
            const DevSlots<T> &D = slots_[3 * side + c];
            SlotView<T> &v = p.slot[c];
            v.map = D.map;
            v.rows = D.rows;
            v.g = D.g;
            v.coef = D.coef;
            v.inv = D.inv;
            v.group = D.group;
            v.rec = D.rec;
            v.stride = D.stride;
            v.A = D.A;
            v.amp = D.amp;
            v.P = D.P;
            v.P1 = D.P1;
            v.n = D.n;
        }
        p.grp_np = grp_np_[side];
        p.grp_pool = grp_pool_[side];
        p.pool_c = pool_c_[side];
        p.comp_base = 3 * side;
        p.nunits = (int)side_units_[side].size();
        int foff = 0;
        for (int su = 0; su < p.nunits; ++su)
        {
            int u = side_units_[side][su];
            const DftUnit &U = P_.units[u];
            DftView &d = p.units[su];
            d.comp = U.comp;
            d.is_db = U.is_db ? 1 : 0;
            for (int a = 0; a < 3; ++a)
            {
                d.i0[a] = U.i0[a];
                d.ld[a] = U.ldim[a];
            }
            d.nf = (int)U.freqs.size();
            d.foff = foff;
            foff += d.nf;
            d.npts = U.npoints();
            d.re = dre_[u];
            d.im = dim_[u];
        }
        // sources
        SourceParams<T> &s = srcp_[side];
        s = SourceParams<T>();
        const DevSources &S = src_[side];
        s.npts = S.npts;
        s.comp = S.comp;
        s.lin = S.lin;
        s.off = S.off;
        s.amp = S.amp;
        s.start = S.start;
        s.end = S.end;
        s.width = S.width;
        s.kind = S.kind;
        s.dt = (T)P_.dt;
        for (int c = 0; c < 3; ++c)
        {
            s.f[c] = p.f[c];
            s.slot[c] = p.slot[c];
        }
        s.coef_def = p.coef_def;
        s.grp_np = p.grp_np;
        s.correct = side == 0 ? 1 : 0;
        s.moff = S.moff;
        s.munit = S.munit;
        s.mlin = S.mlin;
        s.nunits = p.nunits;
        for (int su = 0; su < p.nunits; ++su) s.units[su] = p.units[su];
    }
    for (int c = 0; c < 6; ++c) gp_.f[c] = gpe_.f[c] = buf_[cur_][c];
}

template <typename T>
void Engine<T>::compute_bytes()
{
    // Algorithmic (compulsory) bytes of one full time step:
    //  every component point: field read + write;
    //  every (point, transverse axis) with a non-zero CPML c: psi read + write;
    //  every slot with p poles: P and P' read + write per pole;
    //  every monitored point: re + im read + write (fp64) per frequency.
    const double s = sizeof(T);
    double b = 0;
    for (int c = 0; c < 6; ++c)
    {
        int64_t n[3];
        for (int a = 0; a < 3; ++a) n[a] = std::max(0, P_.vhi[c][a] - P_.vlo[c][a] + 1);
        b += 2 * s * (double)(n[0] * n[1] * n[2]);
        if (P_.any_pml)
            for (int t = 0; t < 2; ++t)
            {
                int a = (c % 3 + 1 + t) % 3;
                int q = comp_parity(c, a);
                int64_t cnt = 0;
                for (int i = P_.vlo[c][a]; i <= P_.vhi[c][a]; ++i) cnt += P_.pml_c[a][q][i] != 0;
                int64_t other = 1;
                for (int a2 = 0; a2 < 3; ++a2)
                    if (a2 != a) other *= n[a2];
                b += 2 * s * (double)(cnt * other);
            }
        b += s * 4 * (double)pole_sum_[c];
    }
    pass_bytes_per_step_ = b;
    for (auto &U : P_.units) b += 32.0 * (double)U.npoints() * (double)U.freqs.size();
    bytes_per_step_ = b;
}

template <typename T>
void Engine<T>::set_phases(int side, double t, double (*phase)[2])
{
    // src/dft.cpp:52-53
    int k = 0;
    for (int u : side_units_[side])
        for (double f : P_.units[u].freqs)
        {
            phase[k][0] = std::cos(2 * kPi * f * t);
            phase[k][1] = -std::sin(2 * kPi * f * t);
            ++k;
        }
}

template <typename T>
void Engine<T>::one_step()
{
    const double dt = P_.dt;
    // ---- H half step: sources at t = n dt, DFT at (n + 1/2) dt
    set_phases(1, (ts_ + 0.5) * dt, sp_[1].phase);
    bool h_src_active = false;
    {
        double t = ts_ * dt;
        if (src_[1].npts && !(t > src_[1].max_end))
        {
            srcp_[1].time = t;
            be_->sources(srcp_[1]);
            ++nlaunch_;
            h_src_active = true;
        }
    }
    set_phases(0, (ts_ + 1) * dt, sp_[0].phase);
    if (fused_)
    {
        FusedParams<T> fp;
        fp.h = sp_[1];
        fp.e = sp_[0];
        const int nx = 1 - cur_;
        for (int c = 0; c < 3; ++c)
        {
            fp.ein[c] = buf_[cur_][c];
            fp.hin[c] = buf_[cur_][3 + c];
            fp.eout[c] = buf_[nx][c];
            fp.hout[c] = buf_[nx][3 + c];
            fp.e.f[c] = buf_[nx][c];
            fp.h.f[c] = buf_[nx][3 + c];
            for (int s = 0; s < 2; ++s)
            {
                const bool even = (ts_ % 2) == 0;
                T *a = psi_[3 + c][s], *b = psih_b_[c][s];
                fp.psih_in[c][s] = even ? a : b;
                fp.psih_out[c][s] = even ? b : a;
            }
        }
        fp.wait_ns = P_.fused_wait_ns;
        fp.stall_test = P_.fused_stall_test ? 1 : 0;
        // H pole state: read the buffers of this step's parity, write the others
        bool h_pending = false;
        for (int c = 0; c < 3; ++c)
        {
            DevSlots<T> &D = slots_[3 + c];
            if (!D.Pb) continue;
            SlotView<T> &v = fp.h.slot[c];
            const bool even = (ts_ % 2) == 0;
            v.P = even ? D.P : D.Pb;
            v.P1 = even ? D.P1 : D.P1b;
            v.Po = even ? D.Pb : D.P;
            v.P1o = even ? D.P1b : D.P1;
            h_pending = h_pending || D.A != nullptr;
        }
        for (int c = 0; c < 6; ++c) gph_.f[c] = buf_[nx][c];
        nlaunch_ += be_->fused(fp, gph_.nfaces ? &gph_ : nullptr);
        // the pass reads the H sources waiting at slots with poles without
        // clearing them: clear them once every reader has finished, in the
        // steps whose H sources were active
        if (h_pending && h_src_active)
            for (int c = 3; c < 6; ++c)
                if (slots_[c].A) be_->zero(slots_[c].A, slots_[c].n * sizeof(T));
        cur_ = nx;
        for (int c = 0; c < 3; ++c)
        {
            sp_[0].f[c] = srcp_[0].f[c] = buf_[cur_][c];
            sp_[1].f[c] = srcp_[1].f[c] = buf_[cur_][3 + c];
            sp_[0].o[c] = buf_[cur_][3 + c];
            sp_[1].o[c] = buf_[cur_][c];
        }
        for (int c = 0; c < 6; ++c) gp_.f[c] = gpe_.f[c] = buf_[cur_][c];
    }
    else
    {
        be_->update(sp_[1], false);
        ++nlaunch_;
        if (gp_.nfaces) { be_->ghosts(gp_); ++nlaunch_; }
        be_->update(sp_[0], true);
        ++nlaunch_;
    }
    // ---- E sources at t = (n + 1/2) dt, applied after the E update together
    //      with their share of the E DFT sums
    {
        double t = (ts_ + 0.5) * dt;
        if (src_[0].npts && !(t > src_[0].max_end))
        {
            srcp_[0].time = t;
            std::memcpy(srcp_[0].phase, sp_[0].phase, sizeof(sp_[0].phase));
            be_->sources(srcp_[0]);
            ++nlaunch_;
        }
    }
    // the fused pass filled the H ghost planes of the new level already (no
    // later update touches H): only the E faces are left
    const GhostParams<T> &gend = fused_ ? gpe_ : gp_;
    if (gend.nfaces) { be_->ghosts(gend); ++nlaunch_; }
    ++ts_;
    if (P_.divergence_check > 0 && ts_ % P_.divergence_check == 0) check_finite();
}

template <typename T>
void Engine<T>::check_finite()
{
    // the reference has no such check: a diverging run there carries NaN /
    // infinite values into its outputs; here the run stops with an error
    const T *f[6];
    for (int c = 0; c < 6; ++c) f[c] = buf_[cur_][c];
    ++nlaunch_;
    if (be_->any_nonfinite(f, 6, P_.cells()))
        throw Diverged("the simulation diverged: non-finite field values at time step " + std::to_string(ts_) +
                       " (checked every " + std::to_string(P_.divergence_check) + " steps)");
}

template <typename T>
void Engine<T>::run(const Json &stop)
{
    // Simulation::run, src/simulation.cpp:903-958
    const std::string &type = stop.at("type").str();
    const double dt = P_.dt;
    auto steps_until = [&](double t) {
        int64_t n = ts_;
        while (n * dt < t) ++n;
        return n - ts_;
    };
    if (type == "time")
    {
        step(steps_until(stop.at("time").num()));
        return;
    }
    if (type == "decay")
    {
        // run_until_fields_decayed, src/simulation.cpp:844-901: the probe is
        // sampled after every step and inspected at window ends
        double pt[3];
        for (int a = 0; a < 3; ++a) pt[a] = stop.at("position").at(a).num() / P_.dx2;
        int ctype = ctype_from_name(stop.at("field component").str());
        int comp = comp_from_ctype(ctype);
        double interval = stop.at("time interval examined").num(), decay_by = stop.at("decayed by").num();
        // probe points: Yee3::interp, include/utility.hpp:983-1022
        int base[3];
        for (int a = 0; a < 3; ++a) base[a] = (int)std::floor(pt[a]), base[a] = ((base[a] & 1) ^ ((ctype >> a) & 1)) ? base[a] - 1 : base[a];
        double sx = (pt[0] - base[0]) / 2, sy = (pt[1] - base[1]) / 2, sz = (pt[2] - base[2]) / 2;
        double w[8] = {(1 - sx) * (1 - sy) * (1 - sz), sx * (1 - sy) * (1 - sz), (1 - sx) * sy * (1 - sz), sx * sy * (1 - sz),
                       (1 - sx) * (1 - sy) * sz, sx * (1 - sy) * sz, (1 - sx) * sy * sz, sx * sy * sz};
        std::vector<int64_t> lin;
        std::vector<double> wt;
        bool all_in = true, any = true;
        for (int a = 0; a < 3; ++a)
        {
            all_in = all_in && P_.lo[a] <= base[a] && base[a] + 2 <= P_.hi[a];
            any = any && base[a] <= P_.hi[a] && P_.lo[a] <= base[a] + 2;
        }
        int n = 0;
        for (int k = 0; k < 4; k += 2)
            for (int j = 0; j < 4; j += 2)
                for (int i = 0; i < 4; i += 2, ++n)
                {
                    int q[3] = {base[0] + i, base[1] + j, base[2] + k};
                    bool in = true;
                    for (int a = 0; a < 3; ++a) in = in && q[a] >= P_.lo[a] && q[a] <= P_.hi[a];
                    if (!any || !(all_in || in)) continue;
                    lin.push_back(P_.lin(P_.index_of(0, q[0]), P_.index_of(1, q[1]), P_.index_of(2, q[2])));
                    wt.push_back(w[n]);
                }
        int64_t *dlin = nullptr;
        double *dw = nullptr;
        if (!lin.empty())
        {
            dlin = (int64_t *)be_->alloc(lin.size() * sizeof(int64_t));
            dw = (double *)be_->alloc(wt.size() * sizeof(double));
            be_->h2d(dlin, lin.data(), lin.size() * sizeof(int64_t));
            be_->h2d(dw, wt.data(), wt.size() * sizeof(double));
        }
        auto window = [&](int64_t nsteps, std::vector<double> &vals) {
            ensure_scratch(nsteps);
            for (int64_t s = 0; s < nsteps; ++s)
            {
                one_step();
                if (dlin) { be_->probe(buf_[cur_][comp], dlin, dw, (int)lin.size(), scratch_ + s); ++nlaunch_; }
            }
            vals.assign(nsteps, 0.0);
            if (dlin && nsteps) be_->d2h(vals.data(), scratch_, nsteps * sizeof(double));
        };
        std::vector<double> v;
        double mx = 0;
        window(steps_until(P_.turnoff_time), v);
        for (double x : v) mx = std::max(mx, x * x);
        for (int ext = 1;; ++ext)
        {
            window(steps_until(P_.turnoff_time + ext * interval), v);
            double cur = 0;
            for (double x : v) cur = std::max(cur, x * x);
            if (cur > mx) mx = cur;
            if (!(cur / mx > decay_by)) break;
        }
        if (dlin) { be_->release(dlin); be_->release(dw); }
        return;
    }
    // run_until_dft, src/simulation.cpp:782-842
    double center[3], size[3], p1[3], p2[3];
    for (int a = 0; a < 3; ++a)
    {
        center[a] = stop.at("center").at(a).num();
        size[a] = stop.at("size").at(a).num();
        p1[a] = (center[a] - size[a] / 2) / P_.dx2;
        p2[a] = (center[a] + size[a] / 2) / P_.dx2;
    }
    int ctype = ctype_from_name(stop.at("field component").str());
    double interval = stop.at("time interval examined").num(), var = stop.at("variation").num();
    double freq = stop.at("frequency").num();
    int c1[3], c2[3];
    component_closure(p1, p2, ctype, c1, c2);
    int unit = -1;
    for (size_t u = 0; u < P_.units.size(); ++u)
        if (P_.units[u].ctype == ctype && std::equal(c1, c1 + 3, P_.units[u].c1) && std::equal(c2, c2 + 3, P_.units[u].c2)) unit = (int)u;
    if (unit < 0) throw std::runtime_error("dft is not registered");
    const auto &F = P_.units[unit].freqs;
    auto it = std::lower_bound(F.begin(), F.end(), freq);
    if (it == F.end() || *it != freq) throw std::runtime_error("frequency is not registered");
    const int64_t fi = it - F.begin();
    const int64_t np = P_.units[unit].npoints();
    step(steps_until(P_.turnoff_time));
    for (int ext = 1;; ++ext)
    {
        int64_t nsteps = steps_until(P_.turnoff_time + ext * interval);
        ensure_scratch(nsteps);
        for (int64_t s = 0; s < nsteps; ++s)
        {
            one_step();
            be_->dft_norm(dre_[unit] + fi * np, dim_[unit] + fi * np, np, scratch_ + s);
            ++nlaunch_;
        }
        std::vector<double> v(nsteps);
        if (nsteps) be_->d2h(v.data(), scratch_, nsteps * sizeof(double));
        double mx = std::numeric_limits<double>::min(), mn = std::numeric_limits<double>::max();
        for (double x : v)
        {
            if (x > mx) mx = x;
            if (x < mn) mn = x;
        }
        if (!((mx - mn) / mx > var)) break;
    }
}

template <typename T>
std::vector<OutputGroup> Engine<T>::outputs()
{
    // DFT_Hub::output_fields_collective, src/dft.cpp:273-320
    be_->sync();
    std::vector<OutputGroup> out;
    std::vector<std::vector<double>> re(P_.units.size()), im(P_.units.size());
    for (size_t u = 0; u < P_.units.size(); ++u)
    {
        int64_t n = P_.units[u].npoints() * (int64_t)P_.units[u].freqs.size();
        re[u].resize(n);
        im[u].resize(n);
        if (n)
        {
            be_->d2h(re[u].data(), dre_[u], n * sizeof(double));
            be_->d2h(im[u].data(), dim_[u], n * sizeof(double));
        }
    }
    for (auto &r : P_.requests)
    {
        const DftUnit &U = P_.units[r.unit];
        OutputGroup g;
        g.group = r.group;
        const uint64_t nf = r.freqs.size();
        std::vector<uint64_t> shp = {nf, (uint64_t)U.dim[2], (uint64_t)U.dim[1], (uint64_t)U.dim[0]};
        const uint64_t plane = (uint64_t)U.dim[0] * U.dim[1] * U.dim[2];
        std::vector<double> R(nf * plane, 0.0), I(nf * plane, 0.0);
        const int64_t np = U.npoints();
        if (np)
        {
            int off[3];
            for (int a = 0; a < 3; ++a) off[a] = (U.l1[a] - U.c1[a]) / 2;
            for (uint64_t f = 0; f < nf; ++f)
            {
                auto it = std::lower_bound(U.freqs.begin(), U.freqs.end(), r.freqs[f]);
                if (it == U.freqs.end() || *it != r.freqs[f]) throw std::runtime_error("Frequencies not registered");
                int64_t fi = it - U.freqs.begin();
                for (int k = 0; k < U.ldim[2]; ++k)
                    for (int j = 0; j < U.ldim[1]; ++j)
                        for (int i = 0; i < U.ldim[0]; ++i)
                        {
                            int64_t src = fi * np + ((int64_t)k * U.ldim[1] + j) * U.ldim[0] + i;
                            uint64_t dst = f * plane + ((uint64_t)(k + off[2]) * U.dim[1] + (j + off[1])) * U.dim[0] + (i + off[0]);
                            R[dst] = re[r.unit][src];
                            I[dst] = im[r.unit][src];
                        }
            }
        }
        auto lins = [](double s, double e, int n) {
            std::vector<double> v;
            if (n <= 1) return std::vector<double>{s};
            double st = (e - s) / (n - 1);
            for (int i = 0; i < n; ++i) v.push_back(s + i * st);
            return v;
        };
        g.names = {"real", "imag", "x", "y", "z", "f"};
        g.shapes = {shp, shp, {(uint64_t)U.dim[0]}, {(uint64_t)U.dim[1]}, {(uint64_t)U.dim[2]}, {nf}};
        g.data = {R, I, lins(U.c1[0] * (P_.dx / 2), U.c2[0] * (P_.dx / 2), U.dim[0]),
                  lins(U.c1[1] * (P_.dx / 2), U.c2[1] * (P_.dx / 2), U.dim[1]),
                  lins(U.c1[2] * (P_.dx / 2), U.c2[2] * (P_.dx / 2), U.dim[2]), r.freqs};
        out.push_back(std::move(g));
    }
    for (auto &gi : P_.geom_info)
    {
        OutputGroup g;
        g.group = gi.group;
        g.names = {"x", "y", "z"};
        g.shapes = {{gi.x.size()}, {gi.y.size()}, {gi.z.size()}};
        g.data = {gi.x, gi.y, gi.z};
        out.push_back(std::move(g));
    }
    return out;
}

template <typename T>
void Engine<T>::reset()
{
    const int64_t cells = P_.cells();
    for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 6; ++c)
            if (buf_[b][c]) be_->zero(buf_[b][c], cells * sizeof(T));
    for (int c = 0; c < 6; ++c)
        for (int s = 0; s < 2; ++s)
            if (psi_[c][s]) be_->zero(psi_[c][s], cells * sizeof(T));
    for (int c = 0; c < 3; ++c)
        for (int s = 0; s < 2; ++s)
            if (psih_b_[c][s]) be_->zero(psih_b_[c][s], cells * sizeof(T));
    for (int c = 0; c < 6; ++c)
    {
        DevSlots<T> &D = slots_[c];
        if (D.A) be_->zero(D.A, D.n * sizeof(T));
        if (D.P) be_->zero(D.P, D.n * D.stride * sizeof(T));
        if (D.P1) be_->zero(D.P1, D.n * D.stride * sizeof(T));
        if (D.Pb) be_->zero(D.Pb, D.n * D.stride * sizeof(T));
        if (D.P1b) be_->zero(D.P1b, D.n * D.stride * sizeof(T));
    }
    for (size_t u = 0; u < P_.units.size(); ++u)
    {
        int64_t n = P_.units[u].npoints() * (int64_t)P_.units[u].freqs.size();
        if (n)
        {
            be_->zero(dre_[u], n * sizeof(double));
            be_->zero(dim_[u], n * sizeof(double));
        }
    }
    cur_ = 0;
    ts_ = 0;
    be_->clear_error();
    bind_params();
}

template <typename T>
void Engine<T>::set_density(const std::string &dataset, const double *rho, uint64_t n)
{
    bool found = false;
    for (auto &g : P_.geoms)
        if ((g.type == Geometry::TWO_MEDIUM_BOX || g.type == Geometry::GENERAL_MEDIUM_BOX) && g.density_dataset == dataset)
        {
            if (n != g.rho.size()) throw std::runtime_error("density size does not match the box dimension");
            g.rho.assign(rho, rho + n);
            found = true;
        }
    if (!found) throw std::runtime_error("no density box uses dataset '" + dataset + "'");
    be_->sync();
    // rasterised again where the handle rasterised first
    if (device_media_) init_media_device();
    else
    {
        rasterize_media(P_);
        init_media();
    }
    alloc_fused_pole_state();
    reset();
    compute_bytes();
}
template <typename T>
void Engine<T>::set_source_data(const std::map<std::string, std::vector<double>> &data)
{
    for (auto &kv : data)
    {
        auto it = P_.source_data.find(kv.first);
        if (it == P_.source_data.end())
            throw std::runtime_error("no inhomogeneous source uses dataset '" + kv.first + "'");
        if (kv.second.size() != it->second.size())
            throw std::runtime_error("dataset '" + kv.first + "' has " + std::to_string(kv.second.size()) +
                                     " values, the source uses " + std::to_string(it->second.size()));
    }
    for (auto &kv : data) P_.source_data[kv.first] = kv.second;
    be_->sync();
    rebuild_sources(P_);
    for (void *p : src_allocs_) be_->release(p);
    src_allocs_.clear();
    init_sources();
    reset();
}
} // namespace

std::unique_ptr<EngineBase> make_engine(Plan &&plan, Backend *be)
{
    if (plan.precision_fp32) return std::unique_ptr<EngineBase>(new Engine<float>(std::move(plan), be));
    return std::unique_ptr<EngineBase>(new Engine<double>(std::move(plan), be));
}
} // namespace ffipg
