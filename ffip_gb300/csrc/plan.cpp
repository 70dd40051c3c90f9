// Host-side set-up: config JSON -> Plan.  Each step cites the part of the
// reference's Simulation::init it reproduces.
#include "plan.hpp"

#include <algorithm>
#include <cmath>
#include <exception>
#include <stdexcept>
#include <thread>

namespace ffipg
{
int ctype_from_name(const std::string &n)
{
    static const std::map<std::string, int> m = {{"Ex", 0b001}, {"Ey", 0b010}, {"Ez", 0b100}, {"Hx", 0b110},
                                                  {"Hy", 0b101}, {"Hz", 0b011}, {"Dx", 0b1001}, {"Dy", 0b1010},
                                                  {"Dz", 0b1100}, {"Bx", 0b1110}, {"By", 0b1101}, {"Bz", 0b1011}};
    auto it = m.find(n);
    if (it == m.end()) throw std::runtime_error("unknown field component '" + n + "'");
    return it->second;
}

int comp_from_ctype(int ctype)
{
    switch (ctype & 7)
    {
    case 0b001: return EX;
    case 0b010: return EY;
    case 0b100: return EZ;
    case 0b110: return HX;
    case 0b101: return HY;
    case 0b011: return HZ;
    }
    throw std::runtime_error("not a field component ctype");
}

void Susceptibility::coefficients(double dt, double &c1, double &c2, double &c3) const
{
    double c0 = 2 * b2 + b1 * dt;
    c1 = (4 * b2 - 2 * b0 * dt * dt) / c0;
    c2 = (-2 * b2 + b1 * dt) / c0;
    c3 = (2 * a0 * dt * dt) / c0;
}

void Susceptibility::increment_coefficients(double dt, double &d1, double &d2, double &c3) const
{
    // c1 + c2 - 1 = (4 b2 - 2 b0 dt^2 - 2 b2 + b1 dt - c0) / c0 = -2 b0 dt^2 / c0
    double c0 = 2 * b2 + b1 * dt;
    d1 = -2 * b0 * dt * dt / c0;
    d2 = (2 * b2 - b1 * dt) / c0;
    c3 = (2 * a0 * dt * dt) / c0;
}

int64_t Plan::yee_cells() const
{
    int64_t n = 1;
    for (int a = 0; a < 3; ++a) n *= std::max(1, (hi[a] - lo[a]) / 2);
    return n;
}

namespace
{
double std_round(double x) { return std::round(x); }  // halves away from zero, as std::round

// get_nearest_int<S,T>, include/utility.hpp:478-498
int nearest_int(int x, int S, int T) { return ((x & 1) ^ T) ? x + S : x; }
int nearest_int_d(double x, int S, int T) { return nearest_int(S == -1 ? (int)std::floor(x) : (int)std::ceil(x), S, T); }

Susceptibility parse_sus(const Json &j)
{
    // src/simulation.cpp:88-100 and factories src/medium.cpp:98-118
    const std::string &t = j.at("type").str();
    Susceptibility s;
    if (t == "Lorentz" || t == "Drude")
    {
        double w = 2 * kPi * j.at("frequency").num();
        s.a0 = w * w;
        s.b0 = (t == "Lorentz") ? w * w : 0.0;
        s.b1 = 2 * kPi * j.at("gamma").num();
        s.b2 = 1;
    }
    else if (t == "Deybe" || t == "Debye")
    {
        s.a0 = 1;
        s.b0 = 1;
        s.b1 = j.at("tau").num();
        s.b2 = 0;
    }
    else
        throw std::runtime_error("unknown susceptibility type '" + t + "'");
    return s;
}

Medium parse_medium(const Json &j)
{
    // json2medium, src/simulation.cpp:58-81 (conductivities default to 0 here)
    Medium m;
    m.epsilon = j.at("epsilon").num();
    m.mu = j.at("mu").num();
    Susceptibility cond;
    cond.a0 = 1;
    cond.b1 = 1;
    double ec = j.num("electric conductivity", 0.0), mc = j.num("magnetic conductivity", 0.0);
    if (ec != 0) { m.e_sus.push_back(cond); m.e_amp.push_back(ec); }
    if (mc != 0) { m.m_sus.push_back(cond); m.m_amp.push_back(mc); }
    if (j.has("electric susceptibility"))
        for (auto &s : j.at("electric susceptibility").items()) { m.e_sus.push_back(parse_sus(s)); m.e_amp.push_back(s.at("amplitude").num()); }
    if (j.has("magnetic susceptibility"))
        for (auto &s : j.at("magnetic susceptibility").items()) { m.m_sus.push_back(parse_sus(s)); m.m_amp.push_back(s.at("amplitude").num()); }
    return m;
}

void add_to_pool(Plan &p, const Medium &m)
{
    // Structure::add_to_material_pool, src/structure.cpp:95-124
    for (auto &s : m.e_sus)
        if (std::find(p.pool[0].begin(), p.pool[0].end(), s) == p.pool[0].end()) p.pool[0].push_back(s);
    for (auto &s : m.m_sus)
        if (std::find(p.pool[1].begin(), p.pool[1].end(), s) == p.pool[1].end()) p.pool[1].push_back(s);
}

PoolMedium to_pool(const Plan &p, const Medium &m)
{
    // Structure::get_abstract_medium, src/structure.cpp:126-153
    PoolMedium r;
    r.epsilon = m.epsilon;
    r.mu = m.mu;
    r.e_amp.assign(p.pool[0].size(), 0.0);
    r.m_amp.assign(p.pool[1].size(), 0.0);
    for (size_t i = 0; i < m.e_sus.size(); ++i)
        for (size_t j = 0; j < p.pool[0].size(); ++j)
            if (p.pool[0][j] == m.e_sus[i]) { r.e_amp[j] = m.e_amp[i]; break; }
    for (size_t i = 0; i < m.m_sus.size(); ++i)
        for (size_t j = 0; j < p.pool[1].size(); ++j)
            if (p.pool[1][j] == m.m_sus[i]) { r.m_amp[j] = m.m_amp[i]; break; }
    return r;
}

std::vector<double> get_dataset(const std::map<std::string, Dataset> &ds, const std::string &name)
{
    auto it = ds.find(name);
    if (it == ds.end()) throw std::runtime_error("dataset not provided: '" + name + "'");
    return std::vector<double>(it->second.data, it->second.data + it->second.n);
}

// one axis of interpn (include/utility.hpp:670-697): returns the number of
// terms (0, 1 or 2) with their indices and weights, in the reference's order
int interp_axis(double q, int n, int idx[2], double w[2])
{
    if (n == 1) { idx[0] = 0; w[0] = 1; return -1; }  // dimension ignored
    if (q <= 0)
    {
        if (q <= -1) return 0;
        idx[0] = 0; w[0] = q + 1;
        return 1;
    }
    if (q >= n - 1)
    {
        if (q >= n) return 0;
        idx[0] = n - 1; w[0] = (double)n - q;
        return 1;
    }
    size_t i = (size_t)q;
    double tx = q - (double)i;
    idx[0] = (int)i + 1; w[0] = tx;
    idx[1] = (int)i; w[1] = 1 - tx;
    return 2;
}
} // namespace

double Geometry::density_at(double x, double y, double z) const
{
    // Two_Medium_Box::get_medium argument, src/geometry.cpp:68-76; interpn<3>(dz, dy, dx)
    double zq = (z - p1[2]) / (p2[2] - p1[2]) * (dim[2] - 1);
    double yq = (y - p1[1]) / (p2[1] - p1[1]) * (dim[1] - 1);
    double xq = (x - p1[0]) / (p2[0] - p1[0]) * (dim[0] - 1);
    int iz[2], iy[2], ix[2];
    double wz[2], wy[2], wx[2];
    int nz = interp_axis(zq, dim[2], iz, wz);
    int ny = interp_axis(yq, dim[1], iy, wy);
    int nxt = interp_axis(xq, dim[0], ix, wx);
    auto at = [&](int k, int j, int i) { return rho[((size_t)k * dim[1] + j) * dim[0] + i]; };
    auto lx = [&](int k, int j) -> double {
        if (nxt == -1) return at(k, j, 0);
        if (nxt == 0) return 0.0;
        if (nxt == 1) return wx[0] * at(k, j, ix[0]);
        return wx[0] * at(k, j, ix[0]) + wx[1] * at(k, j, ix[1]);
    };
    auto ly = [&](int k) -> double {
        if (ny == -1) return lx(k, 0);
        if (ny == 0) return 0.0;
        if (ny == 1) return wy[0] * lx(k, iy[0]);
        return wy[0] * lx(k, iy[0]) + wy[1] * lx(k, iy[1]);
    };
    if (nz == -1) return ly(0);
    if (nz == 0) return 0.0;
    if (nz == 1) return wz[0] * ly(iz[0]);
    return wz[0] * ly(iz[0]) + wz[1] * ly(iz[1]);
}

bool Geometry::inside(double x, double y, double z) const
{
    if (type == SPHERE)
    {
        // CGAL Sphere_3::has_on_bounded_side (strict), src/geometry.cpp:13-15
        double dx = x - center[0], dy = y - center[1], dz = z - center[2];
        return dx * dx + dy * dy + dz * dz < radius * radius;
    }
    // CGAL Iso_cuboid_3::has_on_bounded_side (strict)
    return x > lo[0] && x < hi[0] && y > lo[1] && y < hi[1] && z > lo[2] && z < hi[2];
}

void Geometry::bbox(double blo[3], double bhi[3]) const
{
    for (int a = 0; a < 3; ++a)
    {
        if (type == SPHERE) { blo[a] = center[a] - radius; bhi[a] = center[a] + radius; }
        else { blo[a] = lo[a]; bhi[a] = hi[a]; }
    }
}

PoolMedium Geometry::medium_at(double x, double y, double z) const
{
    if (type == BOX || type == SPHERE) return medium;
    double v = density_at(x, y, z);
    if (type == TWO_MEDIUM_BOX)
    {
        // m1 * val + m2 * (1 - val), src/geometry.cpp:75
        PoolMedium r;
        r.epsilon = medium1.epsilon * v + medium2.epsilon * (1 - v);
        r.mu = medium1.mu * v + medium2.mu * (1 - v);
        r.e_amp.resize(medium1.e_amp.size());
        r.m_amp.resize(medium1.m_amp.size());
        for (size_t i = 0; i < r.e_amp.size(); ++i) r.e_amp[i] = medium1.e_amp[i] * v + medium2.e_amp[i] * (1 - v);
        for (size_t i = 0; i < r.m_amp.size(); ++i) r.m_amp[i] = medium1.m_amp[i] * v + medium2.m_amp[i] * (1 - v);
        return r;
    }
    // General_Medium_Box, src/geometry.cpp:98-107: 1-D lookup over rho_fun
    double q = (v - rho_fun.front()) / (rho_fun.back() - rho_fun.front()) * (double)(rho_fun.size() - 1);
    int idx[2];
    double w[2];
    int nt = interp_axis(q, (int)rho_fun.size(), idx, w);
    PoolMedium r;
    const PoolMedium &ref = medium_fun.front();
    r.e_amp.assign(ref.e_amp.size(), 0.0);
    r.m_amp.assign(ref.m_amp.size(), 0.0);
    if (nt == -1) return medium_fun[0];
    for (int t = 0; t < nt; ++t)
    {
        const PoolMedium &m = medium_fun[idx[t]];
        if (t == 0)
        {
            r.epsilon = w[0] * m.epsilon;
            r.mu = w[0] * m.mu;
            for (size_t i = 0; i < r.e_amp.size(); ++i) r.e_amp[i] = w[0] * m.e_amp[i];
            for (size_t i = 0; i < r.m_amp.size(); ++i) r.m_amp[i] = w[0] * m.m_amp[i];
        }
        else
        {
            r.epsilon = r.epsilon + w[1] * m.epsilon;
            r.mu = r.mu + w[1] * m.mu;
            for (size_t i = 0; i < r.e_amp.size(); ++i) r.e_amp[i] = r.e_amp[i] + w[1] * m.e_amp[i];
            for (size_t i = 0; i < r.m_amp.size(); ++i) r.m_amp[i] = r.m_amp[i] + w[1] * m.m_amp[i];
        }
    }
    return r;
}

void component_closure(const double p1[3], const double p2[3], int ctype, int c1[3], int c2[3])
{
    for (int a = 0; a < 3; ++a)
    {
        int T = (ctype >> a) & 1;
        c1[a] = nearest_int_d(p1[a], -1, T);
        c2[a] = nearest_int_d(p2[a], +1, T);
    }
}

namespace
{
void set_grid(Plan &p)
{
    for (int a = 0; a < 3; ++a)
    {
        p.o[a] = (p.lo[a] & 1) ? p.lo[a] - 1 : p.lo[a];
        p.M[a] = p.index_of(a, p.hi[a] + 1) + 1;
    }
    // 32 elements per row unit: 128 B rows in fp32, 256 B in fp64
    p.Mx_pad = (p.M[0] + 31) / 32 * 32;
    for (int c = 0; c < 6; ++c)
        for (int a = 0; a < 3; ++a)
        {
            int par = comp_parity(c, a);
            int first = ((p.lo[a] & 1) == par) ? p.lo[a] : p.lo[a] + 1;
            int last = ((p.hi[a] & 1) == par) ? p.hi[a] : p.hi[a] - 1;
            p.vlo[c][a] = p.index_of(a, first);
            p.vhi[c][a] = first <= last ? p.index_of(a, last) : p.vlo[c][a] - 1;
        }
}

void set_pmls(Plan &p, const Json &pmls)
{
    // Simulation::set_pmls, src/simulation.cpp:655-726; PML::get_*, src/fields.cpp:488-506
    std::vector<double> k[3], b[3], c[3];
    int sdim[3];
    for (int a = 0; a < 3; ++a)
    {
        sdim[a] = p.hi[a] - p.lo[a] + 1;
        k[a].assign(sdim[a], 1.0);
        b[a].assign(sdim[a], 0.0);
        c[a].assign(sdim[a], 0.0);
    }
    const double dt = p.dt, dx2 = p.dx2;
    for (auto &e : pmls.items())
    {
        double d = e.at("thickness").num(), kmax = e.at("k max").num(), smax = e.at("sigma max").num();
        int m = e.at("order").integer();
        int dir0 = 0, dir1 = 2, side0 = -1, side1 = 1;
        if (e.has("direction"))
        {
            const std::string &s = e.at("direction").str();
            dir0 = dir1 = (s == "x") ? 0 : (s == "y") ? 1 : (s == "z") ? 2 : -1;
            if (dir0 < 0) throw std::runtime_error("bad PML direction '" + s + "'");
        }
        if (e.has("side"))
        {
            const std::string &s = e.at("side").str();
            side0 = side1 = (s == "positive") ? 1 : (s == "negative") ? -1 : 0;
            if (side0 == 0) throw std::runtime_error("bad PML side '" + s + "'");
        }
        auto sigma = [&](double x) { return std::pow(x / d, m) * smax; };
        auto kk = [&](double x) { return 1 + (kmax - 1) * std::pow(x / d, m); };
        auto bb = [&](double x) { return std::exp(-sigma(x) / kk(x) * dt); };
        auto cc = [&](double x) { return 1 / kk(x) * (bb(x) - 1); };
        for (int dir = dir0; dir <= dir1; ++dir)
            for (int side = side0; side <= side1; side += 2)
                for (int i = p.lo[dir]; i <= p.hi[dir]; ++i)
                {
                    double x;
                    if (side == 1 && (i * dx2 >= p.sim_size[dir] / 2 - d)) x = i * dx2 - (p.sim_size[dir] / 2 - d);
                    else if (side == -1 && (i * dx2 <= -p.sim_size[dir] / 2 + d)) x = -p.sim_size[dir] / 2 + d - i * dx2;
                    else continue;
                    int idx = i - p.lo[dir];
                    k[dir][idx] = kk(x);
                    b[dir][idx] = bb(x);
                    c[dir][idx] = cc(x);
                }
    }
    // re-index per parity over array positions
    p.any_pml = false;
    for (int a = 0; a < 3; ++a)
        for (int par = 0; par < 2; ++par)
        {
            p.pml_k[a][par].assign(p.M[a], 1.0);
            p.pml_b[a][par].assign(p.M[a], 0.0);
            p.pml_c[a][par].assign(p.M[a], 0.0);
            for (int i = 0; i < p.M[a]; ++i)
            {
                int crd = p.coord_of(a, i, par);
                if (crd < p.lo[a] || crd > p.hi[a]) continue;
                p.pml_k[a][par][i] = k[a][crd - p.lo[a]];
                p.pml_b[a][par][i] = b[a][crd - p.lo[a]];
                p.pml_c[a][par][i] = c[a][crd - p.lo[a]];
                if (p.pml_c[a][par][i] != 0) p.any_pml = true;
            }
        }
}

Geometry build_geometry(Plan &p, const Json &g, const std::map<std::string, Dataset> &ds)
{
    // Simulation::build_geometry_from_json, src/simulation.cpp:402-518
    Geometry geo;
    const std::string &t = g.at("type").str();
    const double dx2 = p.dx2;
    auto vec3 = [&](const Json &j, double out[3]) {
        for (int a = 0; a < 3; ++a) out[a] = j.at(a).num() / dx2;
    };
    if (t == "box" || t == "sphere")
    {
        geo.type = (t == "box") ? Geometry::BOX : Geometry::SPHERE;
        geo.medium = to_pool(p, parse_medium(g.at("medium")));
        vec3(g.at("center"), geo.center);
        if (t == "box") vec3(g.at("size"), geo.size);
        else geo.radius = g.at("radius").num() / dx2;
    }
    else if (t == "two medium box" || t == "general medium box")
    {
        vec3(g.at("center"), geo.center);
        vec3(g.at("size"), geo.size);
        for (int a = 0; a < 3; ++a) geo.dim[a] = g.at("dimension").at(a).integer();
        geo.density_dataset = g.at("density dataset").str();
        geo.rho = get_dataset(ds, geo.density_dataset);
        if ((int64_t)geo.rho.size() != (int64_t)geo.dim[0] * geo.dim[1] * geo.dim[2])
            throw std::runtime_error("density dataset '" + geo.density_dataset + "' does not match the box dimension");
        if (t == "two medium box")
        {
            geo.type = Geometry::TWO_MEDIUM_BOX;
            geo.medium1 = to_pool(p, parse_medium(g.at("medium1")));
            geo.medium2 = to_pool(p, parse_medium(g.at("medium2")));
        }
        else
        {
            geo.type = Geometry::GENERAL_MEDIUM_BOX;
            Medium med = parse_medium(g.at("medium"));
            geo.rho_fun = get_dataset(ds, g.at("density function dataset").str());
            auto eps = get_dataset(ds, g.at("epsilon dataset").str());
            auto mu = get_dataset(ds, g.at("mu dataset").str());
            auto ea = get_dataset(ds, g.at("electric susceptibility amplitudes dataset").str());
            auto ma = get_dataset(ds, g.at("magnetic susceptibility amplitudes dataset").str());
            if (geo.rho_fun.size() < 1 || eps.size() != geo.rho_fun.size())
                throw std::runtime_error("general medium box: density function and epsilon datasets must match");
            for (size_t i = 0; i < eps.size(); ++i)
            {
                Medium m = med;
                m.epsilon = eps[i];
                m.mu = i < mu.size() ? mu[i] : 1.0;
                for (size_t j = 0; j < m.e_amp.size(); ++j) m.e_amp[j] = ea.at(i * med.e_amp.size() + j);
                for (size_t j = 0; j < m.m_amp.size(); ++j) m.m_amp[j] = ma.at(i * med.m_amp.size() + j);
                geo.medium_fun.push_back(to_pool(p, m));
            }
        }
    }
    else
        throw std::runtime_error("unknown geometry type '" + t + "'");
    for (int a = 0; a < 3; ++a)
    {
        geo.p1[a] = geo.center[a] - geo.size[a] / 2;
        geo.p2[a] = geo.center[a] + geo.size[a] / 2;
        geo.lo[a] = std::min(geo.p1[a], geo.p2[a]);
        geo.hi[a] = std::max(geo.p1[a], geo.p2[a]);
    }
    return geo;
}

void add_dipole(Plan &p, const double pos[3], int ctype, double amp, double start, double freq, double cutoff, int kind)
{
    // Fields::add_dipole_source_gaussian1/2, src/fields.cpp:183-232
    amp = -amp;
    int base[3];
    for (int a = 0; a < 3; ++a) base[a] = nearest_int_d(pos[a], -1, (ctype >> a) & 1);
    double sx = (pos[0] - base[0]) / 2, sy = (pos[1] - base[1]) / 2, sz = (pos[2] - base[2]) / 2;
    double w[8] = {(1 - sx) * (1 - sy) * (1 - sz), sx * (1 - sy) * (1 - sz), (1 - sx) * sy * (1 - sz), sx * sy * (1 - sz),
                   (1 - sx) * (1 - sy) * sz, sx * (1 - sy) * sz, (1 - sx) * sy * sz, sx * sy * sz};
    double width = (kind == 1) ? 1 / (2 * kPi * freq) : std::sqrt(2.0) / (2 * kPi * freq);
    double end = start + 2 * width * cutoff;
    if (end > p.turnoff_time) p.turnoff_time = end;
    const int side = ctype_is_e(ctype) ? 0 : 1;
    const int comp = comp_from_ctype(ctype);
    int n = 0;
    for (int k = 0; k < 4; k += 2)
        for (int j = 0; j < 4; j += 2)
            for (int i = 0; i < 4; i += 2, ++n)
            {
                int q[3] = {base[0] + i, base[1] + j, base[2] + k};
                bool in = true;
                for (int a = 0; a < 3; ++a) in = in && q[a] >= p.lo[a] && q[a] <= p.hi[a];
                // Gaussian1 keeps corners with weight > 1e-4 (src/fields.cpp:203).
                // The reference's Gaussian2 path mis-steps its weight index
                // (src/fields.cpp:222-230, reads past the weight array); here
                // both kinds use the corner's own weight.
                if (!in || (kind == 1 && !(w[n] > 1e-4))) continue;
                Dipole d;
                d.comp = comp;
                d.lin = p.lin(p.index_of(0, q[0]), p.index_of(1, q[1]), p.index_of(2, q[2]));
                d.amp = amp * w[n];
                d.start = start;
                d.end = end;
                d.width = width;
                d.kind = kind;
                p.dipoles[side].push_back(d);
            }
}

int func_kind(const Json &f)
{
    const std::string &t = f.at("type").str();
    if (t == "Gaussian1") return 1;
    if (t == "Gaussian2") return 2;
    return 0;  // the reference prints "Source function type not supported" and skips
}

void set_volume_source(Plan &p, const Json &s)
{
    // Simulation::set_volume_source, src/simulation.cpp:235-282
    double center[3], size[3], p1[3], dlen[3];
    int count[3];
    for (int a = 0; a < 3; ++a)
    {
        center[a] = s.at("center").at(a).num() / p.dx2;
        size[a] = s.at("size").at(a).num() / p.dx2;
    }
    double amp = s.at("amplitude").num();
    int ctype = ctype_from_name(s.at("field component").str());
    const Json &f = s.at("function");
    int kind = func_kind(f);
    double freq = f.at("frequency").num(), cutoff = f.at("cutoff").num(), st = f.at("start time").num();
    for (int a = 0; a < 3; ++a)
    {
        p1[a] = center[a] - size[a] / 2;
        count[a] = (int)std_round(size[a] / 2);
    }
    for (int a = 0; a < 3; ++a)
    {
        if (count[a] != 0)
        {
            dlen[a] = size[a] / count[a];
            amp *= dlen[a] / 2;
        }
        else
            dlen[a] = 0;
    }
    if (!kind) return;
    for (int k = 0; k <= count[2]; ++k)
        for (int j = 0; j <= count[1]; ++j)
            for (int i = 0; i <= count[0]; ++i)
            {
                double q[3] = {p1[0] + i * dlen[0], p1[1] + j * dlen[1], p1[2] + k * dlen[2]};
                add_dipole(p, q, ctype, amp, st, freq, cutoff, kind);
            }
}

void set_inhom_source(Plan &p, const Json &s, const std::map<std::string, Dataset> &ds)
{
    // Simulation::set_inhom_source, src/simulation.cpp:284-336
    double center[3], size[3], p1[3], dlen[3];
    int dim[3];
    for (int a = 0; a < 3; ++a)
    {
        center[a] = s.at("center").at(a).num() / p.dx2;
        size[a] = s.at("size").at(a).num() / p.dx2;
        dim[a] = s.at("dimension").at(a).integer();
        p1[a] = center[a] - size[a] / 2;
        dlen[a] = dim[a] > 1 ? size[a] / (dim[a] - 1) : 0.0;
    }
    auto amp = get_dataset(ds, s.at("amplitude dataset").str());
    auto phase = get_dataset(ds, s.at("phase dataset").str());
    size_t npts = (size_t)std::max(dim[0], 0) * std::max(dim[1], 0) * std::max(dim[2], 0);
    if (amp.size() < npts || phase.size() < npts)
        throw std::runtime_error("inhomogeneous source: amplitude/phase datasets smaller than the source dimension");
    int ctype = ctype_from_name(s.at("field component").str());
    double fcen = s.at("frequency").num();
    const Json &f = s.at("function");
    int kind = func_kind(f);
    double freq = f.at("frequency").num(), cutoff = f.at("cutoff").num(), st = f.at("start time").num();
    if (!kind) return;
    size_t n = 0;
    for (int k = 0; k < dim[2]; ++k)
        for (int j = 0; j < dim[1]; ++j)
            for (int i = 0; i < dim[0]; ++i, ++n)
            {
                double q[3] = {p1[0] + i * dlen[0], p1[1] + j * dlen[1], p1[2] + k * dlen[2]};
                add_dipole(p, q, ctype, amp[n], st - phase[n] / (2 * kPi * fcen), freq, cutoff, kind);
            }
}

void set_fields_output(Plan &p, const Json &outs)
{
    // Volume_Fields_DFT (src/simulation.cpp:103-118), DFT_Hub::register_volume_dft
    // (src/dft.cpp:253-271), DFT_Unit::set_local_region (src/dft.cpp:163-180)
    for (auto &o : outs.items())
    {
        if (o.at("type").str() != "volume fields dft") continue;
        double center[3], size[3], p1[3], p2[3];
        for (int a = 0; a < 3; ++a)
        {
            center[a] = o.at("center").at(a).num() / (p.dx / 2);
            size[a] = o.at("size").at(a).num() / (p.dx / 2);
            p1[a] = center[a] - size[a] / 2;
            p2[a] = center[a] + size[a] / 2;
        }
        std::vector<double> freqs;
        for (auto &f : o.at("frequency").items()) freqs.push_back(f.num());
        int ctype = ctype_from_name(o.at("field component").str());
        int c1[3], c2[3];
        component_closure(p1, p2, ctype, c1, c2);
        int found = -1;
        for (size_t u = 0; u < p.units.size(); ++u)
        {
            const DftUnit &U = p.units[u];
            if (U.ctype == ctype && std::equal(c1, c1 + 3, U.c1) && std::equal(c2, c2 + 3, U.c2)) { found = (int)u; break; }
        }
        if (found < 0)
        {
            DftUnit U;
            U.ctype = ctype;
            U.comp = comp_from_ctype(ctype);
            U.is_db = ctype > 7;
            for (int a = 0; a < 3; ++a)
            {
                U.c1[a] = c1[a];
                U.c2[a] = c2[a];
                U.dim[a] = (c2[a] - c1[a]) / 2 + 1;
                if (U.dim[a] < 1) throw std::runtime_error("Invali volume in DFT_Unit constructor");
            }
            bool inter = true;
            for (int a = 0; a < 3; ++a) inter = inter && c1[a] <= p.hi[a] && p.lo[a] <= c2[a];
            if (inter)
            {
                U.has_local = true;
                for (int a = 0; a < 3; ++a)
                {
                    int q1 = std::max(c1[a], p.lo[a]), q2 = std::min(c2[a], p.hi[a]);
                    int T = (ctype >> a) & 1;
                    int l1 = nearest_int(q1, +1, T), l2 = nearest_int(q2, -1, T);
                    U.l1[a] = l1;
                    U.ldim[a] = (l2 - l1) / 2 + 1;
                    if (U.ldim[a] <= 0) U.has_local = false;
                    U.i0[a] = p.index_of(a, l1);
                }
            }
            found = (int)p.units.size();
            p.units.push_back(U);
        }
        for (double f : freqs) p.units[found].freqs.push_back(f);
        DftRequest r;
        r.unit = found;
        r.freqs = freqs;
        r.group = o.at("output group").str();
        p.requests.push_back(r);
    }
    for (auto &U : p.units)
    {
        std::sort(U.freqs.begin(), U.freqs.end());
        U.freqs.erase(std::unique(U.freqs.begin(), U.freqs.end()), U.freqs.end());
    }
}
} // namespace

bool geometry_index_range(const Plan &p, const Geometry &geo, int c, int r0[3], int r1[3])
{
    // the component's points within the geometry's bounding box, one point of
    // margin (the strict inside test decides)
    double blo[3], bhi[3];
    geo.bbox(blo, bhi);
    bool empty = false;
    for (int a = 0; a < 3; ++a)
    {
        int par = comp_parity(c, a);
        int cl = (int)std::floor(blo[a]) - 1, ch = (int)std::ceil(bhi[a]) + 1;
        if ((cl & 1) != par) ++cl;
        if ((ch & 1) != par) --ch;
        r0[a] = std::max(p.index_of(a, cl), p.vlo[c][a]);
        r1[a] = std::min(p.index_of(a, ch), p.vhi[c][a]);
        if (r0[a] > r1[a]) empty = true;
    }
    return !empty;
}

void rasterize_media(Plan &p)
{
    // Structure::set_materials_from_geometry with No_Average,
    // src/structure.cpp:155-249: first geometry (in list order) containing a
    // point decides its medium, else the default medium.  A point becomes a
    // slot when its medium differs from the default's (different g_inf, or
    // any pole amplitude above 1e-4, src/structure.cpp:256-264).
    for (int side = 0; side < 2; ++side)
    {
        p.groups[side].clear();
        p.group_index[side].clear();
    }
    const double tol = 1e-4;
    // phase 1, one host thread per component: the points each geometry owns
    // (the first geometry in list order containing the point), as linear
    // indices within the component's valid box in scan order (k, j, i), with
    // the owning geometry
    std::vector<uint64_t> own_li[6];
    std::vector<int> own_g[6];
    auto own = [&](int c) {
        int n[3], first[3];
        for (int a = 0; a < 3; ++a)
        {
            first[a] = p.vlo[c][a];
            n[a] = std::max(0, p.vhi[c][a] - p.vlo[c][a] + 1);
        }
        const uint64_t total = (uint64_t)n[0] * n[1] * n[2];
        if (!total) return;
        std::vector<uint64_t> taken((total + 63) / 64, 0);
        std::vector<std::pair<uint64_t, int>> list;
        for (size_t g = 0; g < p.geoms.size(); ++g)
        {
            int r0[3], r1[3];
            if (!geometry_index_range(p, p.geoms[g], c, r0, r1)) continue;
            for (int k = r0[2]; k <= r1[2]; ++k)
                for (int j = r0[1]; j <= r1[1]; ++j)
                    for (int i = r0[0]; i <= r1[0]; ++i)
                    {
                        const uint64_t li = ((uint64_t)(k - first[2]) * n[1] + (j - first[1])) * n[0] + (i - first[0]);
                        if ((taken[li >> 6] >> (li & 63)) & 1) continue;
                        double x = p.coord_of(0, i, comp_parity(c, 0)), y = p.coord_of(1, j, comp_parity(c, 1)),
                               z = p.coord_of(2, k, comp_parity(c, 2));
                        if (p.geoms[g].inside(x, y, z))
                        {
                            taken[li >> 6] |= uint64_t(1) << (li & 63);
                            list.emplace_back(li, (int)g);
                        }
                    }
        }
        if (p.geoms.size() > 1) std::sort(list.begin(), list.end());
        own_li[c].resize(list.size());
        own_g[c].resize(list.size());
        for (size_t t = 0; t < list.size(); ++t)
        {
            own_li[c][t] = list[t].first;
            own_g[c][t] = list[t].second;
        }
    };
    {
        std::exception_ptr err[6];
        std::vector<std::thread> th;
        for (int c = 0; c < 6; ++c)
            th.emplace_back([&, c] {
                try
                {
                    own(c);
                }
                catch (...)
                {
                    err[c] = std::current_exception();
                }
            });
        for (auto &t : th) t.join();
        for (auto &e : err)
            if (e) std::rethrow_exception(e);
    }
    // phase 2, components in order (pole groups are numbered by first
    // appearance): slots
    for (int c = 0; c < 6; ++c)
    {
        const int side = c < 3 ? 0 : 1;
        const size_t npool = p.pool[side].size();
        SlotList &sl = p.slots[c];
        sl = SlotList();
        int n[3], first[3];
        for (int a = 0; a < 3; ++a)
        {
            first[a] = p.vlo[c][a];
            n[a] = std::max(0, p.vhi[c][a] - p.vlo[c][a] + 1);
        }
        const uint64_t total = (uint64_t)n[0] * n[1] * n[2];
        if (!total) continue;
        const std::vector<double> &def_amp = side == 0 ? p.default_medium.e_amp : p.default_medium.m_amp;
        const double g_def = p.g_default[side];
        std::vector<int> def_bits;
        for (size_t i = 0; i < npool; ++i)
            if (std::abs(def_amp[i]) > tol) def_bits.push_back((int)i);
        const bool all_slots = !def_bits.empty();
        // the medium of a point: g_inf, its active poles (amplitude above tol)
        // and their amplitudes; homogeneous geometries (boxes, spheres) and
        // the default medium are resolved once, at their first point in scan
        // order, so that pole groups are registered at the same points (and
        // numbered the same) as point by point
        struct PointMedium
        {
            bool ready{false};
            double g{0};
            int nb{0}, grp{-1};
            int bits[kMaxPoles];
            double a[kMaxPoles];
        };
        auto resolve = [&](PointMedium &m, double g, const std::vector<double> &amps) {
            m.g = g;
            m.nb = 0;
            for (size_t q = 0; q < npool && q < amps.size(); ++q)
                if (std::abs(amps[q]) > tol)
                {
                    if (m.nb == kMaxPoles)
                        throw std::runtime_error("a grid point has more than " + std::to_string(kMaxPoles) + " active poles");
                    m.bits[m.nb] = (int)q;
                    m.a[m.nb++] = amps[q];
                }
            m.grp = -1;
            m.ready = true;
        };
        auto group_of = [&](const PointMedium &m) {
            std::vector<int> bits(m.bits, m.bits + m.nb);
            auto it = p.group_index[side].find(bits);
            if (it != p.group_index[side].end()) return it->second;
            const int grp = (int)p.groups[side].size();
            p.group_index[side][bits] = grp;
            PoleGroup pg;
            pg.pool = bits;
            p.groups[side].push_back(pg);
            return grp;
        };
        std::vector<PointMedium> cached(p.geoms.size() + 1);  // per geometry; the last: the default medium
        std::vector<double> amp_flat;                         // active-pole amplitudes of the slots, in slot order
        std::vector<uint8_t> amp_n;                           // their count per slot
        // every point in scan order when the default medium makes slots too,
        // else the owned points only
        const std::vector<uint64_t> &OL = own_li[c];
        const std::vector<int> &OG = own_g[c];
        const uint64_t count = all_slots ? total : OL.size();
        for (uint64_t t = 0, cur = 0; t < count; ++t)
        {
            uint64_t li;
            int gi;
            if (all_slots)
            {
                li = t;
                gi = cur < OL.size() && OL[cur] == li ? OG[cur++] : -1;
            }
            else
            {
                li = OL[t];
                gi = OG[t];
            }
            const int i = (int)(li % n[0]), j = (int)(li / n[0] % n[1]), k = (int)(li / ((uint64_t)n[0] * n[1]));
            PointMedium local;
            PointMedium *m;
            if (gi < 0)
            {
                m = &cached.back();
                if (!m->ready) resolve(*m, g_def, def_amp);
            }
            else
            {
                const Geometry &geo = p.geoms[gi];
                if (geo.type == Geometry::BOX || geo.type == Geometry::SPHERE)
                {
                    m = &cached[gi];
                    if (!m->ready)
                        resolve(*m, side == 0 ? geo.medium.epsilon : geo.medium.mu,
                                side == 0 ? geo.medium.e_amp : geo.medium.m_amp);
                }
                else
                {
                    int ii = i + first[0], jj = j + first[1], kk = k + first[2];
                    const PoolMedium tmp = geo.medium_at(p.coord_of(0, ii, comp_parity(c, 0)),
                                                         p.coord_of(1, jj, comp_parity(c, 1)),
                                                         p.coord_of(2, kk, comp_parity(c, 2)));
                    resolve(local, side == 0 ? tmp.epsilon : tmp.mu, side == 0 ? tmp.e_amp : tmp.m_amp);
                    m = &local;
                }
            }
            if (m->nb == 0 && m->g == g_def) continue;
            if (m->grp < 0) m->grp = group_of(*m);
            sl.lin.push_back(p.lin(i + first[0], j + first[1], k + first[2]));
            sl.g.push_back(m->g);
            sl.group.push_back(m->grp);
            amp_flat.insert(amp_flat.end(), m->a, m->a + m->nb);
            amp_n.push_back((uint8_t)m->nb);
            sl.npole_stride = std::max(sl.npole_stride, m->nb);
        }
        const size_t ns = sl.lin.size();
        sl.any_poles = sl.npole_stride > 0;
        sl.amp.assign((size_t)sl.npole_stride * ns, 0.0);
        for (size_t s = 0, o = 0; s < ns; o += amp_n[s], ++s)
            for (size_t q = 0; q < amp_n[s]; ++q) sl.amp[q * ns + s] = amp_flat[o + q];
    }
}

void build_plan(const Json &cfg, const std::map<std::string, Dataset> &ds, Plan &p)
{
    // scalars, src/simulation.cpp:133-141
    p.courant = cfg.num("courant number", 0.5);
    p.resolution = cfg.at("resolution").num();
    if (!(p.resolution > 0)) throw std::runtime_error("resolution must be positive");
    p.dx = 1 / p.resolution;
    p.dt = p.dx * p.courant;
    p.dx2 = p.dx / 2;
    if (!(p.courant > 0) || p.courant > 1 / std::sqrt(3.0) + 1e-12)
        throw std::runtime_error("courant number must be in (0, 1/sqrt(3)] for a stable 3-D Yee update");
    std::string prec = cfg.str("precision", "fp64");
    if (prec != "fp64" && prec != "fp32") throw std::runtime_error("precision must be \"fp64\" or \"fp32\"");
    p.precision_fp32 = prec == "fp32";
    p.engine = cfg.str("engine", "auto");
    // divergence check every N steps (0: off)
    const double every = cfg.num("divergence check interval", 4096);
    if (!(every >= 0) || every > 1e15 || every != std::floor(every))
        throw std::runtime_error("divergence check interval must be a non-negative whole number of steps");
    p.divergence_check = (int64_t)every;
    // bound of the fused pass's device-side waits, and the test of its
    // timeout path
    const double wait_s = cfg.num("fused wait timeout", 2.0);
    if (!(wait_s > 0) || wait_s > 60) throw std::runtime_error("fused wait timeout must be in (0, 60] seconds");
    p.fused_wait_ns = (uint64_t)(wait_s * 1e9);
    p.fused_stall_test = cfg.num("fused wait test", 0) != 0;
    // set_size, src/simulation.cpp:570-581
    for (int a = 0; a < 3; ++a)
    {
        p.sim_size[a] = cfg.at("size").at(a).num();
        int span = (int)std_round(p.sim_size[a] / p.dx) * 2;
        if (span < 2) throw std::runtime_error("simulation size must be at least one cell along every axis");
        p.lo[a] = -span / 2;
        p.hi[a] = span / 2;
    }
    // read_boundary_conditions, src/simulation.cpp:583-653
    for (int a = 0; a < 3; ++a) p.bc[a][0] = p.bc[a][1] = BC_NONE;
    if (cfg.has("symmetry"))
        for (auto &s : cfg.at("symmetry").items())
        {
            const std::string &d = s.at("direction").str();
            int a = d == "x" ? 0 : d == "y" ? 1 : d == "z" ? 2 : -1;
            if (a < 0) continue;
            p.lo[a] = 0;
            p.bc[a][0] = s.at("phase factor").integer() == 1 ? BC_PMC : BC_PEC;
        }
    if (cfg.has("periodic"))
        for (int a = 0; a < 3; ++a)
            if (cfg.at("periodic").at(a).integer())
            {
                if (p.bc[a][0] == BC_PMC || p.bc[a][0] == BC_PEC) p.bc[a][1] = p.bc[a][0];
                else p.bc[a][0] = p.bc[a][1] = BC_PERIOD;
            }
    set_grid(p);
    // media and pool, src/simulation.cpp:159-175,359-400
    Medium bg;
    if (cfg.has("default material")) bg = parse_medium(cfg.at("default material"));
    p.pool[0].clear();
    p.pool[1].clear();
    add_to_pool(p, bg);
    if (cfg.has("PML")) set_pmls(p, cfg.at("PML"));
    else set_pmls(p, Json());
    std::vector<Json> geoms = cfg.has("geometry") ? cfg.at("geometry").items() : std::vector<Json>();
    for (auto &g : geoms)
    {
        if (g.at("type").str() != "two medium box") add_to_pool(p, parse_medium(g.at("medium")));
        else
        {
            add_to_pool(p, parse_medium(g.at("medium1")));
            add_to_pool(p, parse_medium(g.at("medium2")));
        }
    }
    for (int side = 0; side < 2; ++side)
    {
        p.pool_coef[side].clear();
        for (auto &s : p.pool[side])
        {
            std::array<double, 3> c;
            s.increment_coefficients(p.dt, c[0], c[1], c[2]);
            p.pool_coef[side].push_back(c);
        }
    }
    p.geoms.clear();
    for (auto &g : geoms) p.geoms.push_back(build_geometry(p, g, ds));
    p.default_medium = to_pool(p, bg);
    p.g_default[0] = p.default_medium.epsilon;
    p.g_default[1] = p.default_medium.mu;
    // media on the host here unless the engine's backend rasterises them on
    // the device ("rasterize": "auto" / "device")
    p.rasterize = cfg.str("rasterize", "auto");
    if (p.rasterize != "auto" && p.rasterize != "host" && p.rasterize != "device")
        throw std::runtime_error("rasterize must be \"auto\", \"host\" or \"device\"");
    if (p.rasterize == "host") rasterize_media(p);
    // geometry info request, src/simulation.cpp:190-233 (coordinates pass
    // through a std::vector<int> there, i.e. they are truncated toward zero)
    if (cfg.has("geometry info request"))
        for (auto &r : cfg.at("geometry info request").items())
        {
            GeomInfo gi;
            gi.group = r.at("output group").str();
            int ctype = ctype_from_name(r.at("field component").str());
            int gidx = r.at("geometry index").integer();
            int c = comp_from_ctype(ctype);
            for (int k = p.vlo[c][2]; k <= p.vhi[c][2]; ++k)
                for (int j = p.vlo[c][1]; j <= p.vhi[c][1]; ++j)
                    for (int i = p.vlo[c][0]; i <= p.vhi[c][0]; ++i)
                    {
                        double x = p.coord_of(0, i, comp_parity(c, 0)), y = p.coord_of(1, j, comp_parity(c, 1)),
                               z = p.coord_of(2, k, comp_parity(c, 2));
                        int owner = -1;
                        for (size_t g = 0; g < p.geoms.size(); ++g)
                            if (p.geoms[g].inside(x, y, z)) { owner = (int)g; break; }
                        if (owner != gidx) continue;
                        gi.x.push_back((double)(int)(x * p.dx2));
                        gi.y.push_back((double)(int)(y * p.dx2));
                        gi.z.push_back((double)(int)(z * p.dx2));
                    }
            p.geom_info.push_back(gi);
        }
    // sources, src/simulation.cpp:338-357
    p.has_sources = cfg.has("sources");
    p.source_data.clear();
    if (p.has_sources)
    {
        p.sources_cfg = cfg.at("sources");
        for (auto &s : p.sources_cfg.items())
            if (s.at("type").str() == "inhomogeneous source")
                for (const char *key : {"amplitude dataset", "phase dataset"})
                {
                    const std::string &name = s.at(key).str();
                    p.source_data[name] = get_dataset(ds, name);
                }
    }
    rebuild_sources(p);
    if (cfg.has("fields output")) set_fields_output(p, cfg.at("fields output"));
    if (cfg.has("stop condition"))
    {
        p.stop = cfg.at("stop condition");
        p.has_stop = true;
    }
}
void rebuild_sources(Plan &p)
{
    p.dipoles[0].clear();
    p.dipoles[1].clear();
    p.turnoff_time = 0;
    if (!p.has_sources) return;
    std::map<std::string, Dataset> ds;
    for (auto &kv : p.source_data) ds[kv.first] = Dataset{kv.second.data(), kv.second.size()};
    for (auto &s : p.sources_cfg.items())
    {
        const std::string &t = s.at("type").str();
        if (t == "volume source") set_volume_source(p, s);
        else if (t == "inhomogeneous source") set_inhom_source(p, s, ds);
        else throw std::runtime_error("unknown source type '" + t + "'");
    }
}
} // namespace ffipg
