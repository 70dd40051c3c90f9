// Host-side set-up of one simulation: reads the config JSON (the schema of
// ffip's run_sim_json, src/simulation.cpp:127-188) and produces everything the
// device stepper needs, laid out for the GPU.
//
// Grid layout.  The reference works on a doubled grid (integer coordinate =
// 2*x/dx) in which all six components interleave (include/utility.hpp:48-64,
// 907-1023).  Here every component gets its own dense array, all six with the
// same shape (Mx_pad, My, Mz), x fastest.  Along an axis whose doubled range
// is [lo, hi], let o = lo rounded down to even and f the axis's first index
// (kXFirst along x, 1 along y and z); array index i holds the
// coordinate o + 2(i-f) (even-parity components) or o + 2(i-f) + 1 (odd).
// With that convention an even-parity point at index i has its odd neighbours
// at i-1 and i, and an odd-parity point has its even neighbours at i and i+1,
// whatever lo is.  Array positions that hold no grid point of a component
// (including the reference's one-point ghost layer) stay zero, which is the
// reference's "None" boundary; PEC/PMC/periodic ghosts are filled after each
// half step like Fields::sync_boundary (src/fields.cpp:327-482).
#pragma once
#include <array>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "json.hpp"

namespace ffipg
{
constexpr double kPi = 3.141592653589793e+00;  // src/utility.cpp:5
constexpr int kMaxPoles = 8;                    // poles per grid point in one slot
// first array index along x that holds grid points: rows start on a
// 128-byte boundary and the fused pass's tiles start at index kXFirst + 32 u,
// so that every tile's TMA box (kXFirst elements to the left of the tile) is
// 16-byte aligned and the pairs of points that a thread loads and stores as
// one vector are 8-byte aligned
#ifndef FFIP_XFIRST
#define FFIP_XFIRST 2
#endif
constexpr int kXFirst = FFIP_XFIRST;

enum Comp { EX = 0, EY = 1, EZ = 2, HX = 3, HY = 4, HZ = 5 };
enum BC { BC_PEC = 0, BC_PMC = 1, BC_NONE = 2, BC_SYNC = 3, BC_PERIOD = 4 };

// doubled-grid parity bits of each component (include/utility.hpp:48-64)
constexpr int kCtype[6] = {0b001, 0b010, 0b100, 0b110, 0b101, 0b011};
inline int comp_parity(int c, int a) { return (kCtype[c] >> a) & 1; }
inline int comp_dir(int c) { return c % 3; }  // direction x3 of the component
int ctype_from_name(const std::string &name);  // "Ex".."Bz" -> 4-bit ctype
int comp_from_ctype(int ctype);                // low 3 bits -> Comp
inline bool ctype_is_e(int ctype)
{
    int b = ctype & 7;
    return b == 1 || b == 2 || b == 4;
}

struct Susceptibility  // (a0 + a1 jw) / (b0 + b1 jw - b2 w^2), include/medium.hpp:127-134
{
    double a0{0}, a1{0}, b0{0}, b1{0}, b2{0};
    bool operator==(const Susceptibility &o) const { return a0 == o.a0 && a1 == o.a1 && b0 == o.b0 && b1 == o.b1 && b2 == o.b2; }
    // Abstract_Susceptibility, src/medium.cpp:24-31
    void coefficients(double dt, double &c1, double &c2, double &c3) const;
    // the same recurrence in increment form: d1 = c1 + c2 - 1, d2 = -c2
    // (derived symbolically so that a Drude pole gets d1 = 0 exactly)
    void increment_coefficients(double dt, double &d1, double &d2, double &c3) const;
};

struct Medium
{
    double epsilon{1}, mu{1};
    std::vector<Susceptibility> e_sus, m_sus;
    std::vector<double> e_amp, m_amp;
};

// medium expressed over the susceptibility pool (Abstract_Medium)
struct PoolMedium
{
    double epsilon{0}, mu{0};
    std::vector<double> e_amp, m_amp;
};

struct Geometry
{
    enum Type { BOX, SPHERE, TWO_MEDIUM_BOX, GENERAL_MEDIUM_BOX } type{BOX};
    // all positions in doubled-grid units
    double center[3]{0, 0, 0}, size[3]{0, 0, 0}, radius{0};
    double lo[3]{0, 0, 0}, hi[3]{0, 0, 0};  // strict inside test bounds (boxes)
    double p1[3]{0, 0, 0}, p2[3]{0, 0, 0};  // center -/+ size/2 (density grid corners)
    int dim[3]{1, 1, 1};
    PoolMedium medium, medium1, medium2;
    std::vector<double> rho, rho_fun;
    std::vector<PoolMedium> medium_fun;
    std::string density_dataset;
    bool inside(double x, double y, double z) const;
    // medium at a doubled-grid position (src/geometry.cpp:21-107)
    PoolMedium medium_at(double x, double y, double z) const;
    double density_at(double x, double y, double z) const;
    void bbox(double lo_out[3], double hi_out[3]) const;
};

struct Dipole
{
    int comp;
    int64_t lin;  // linear index in the component array
    double amp, start, end, width;
    int kind;     // 1 = Gaussian1, 2 = Gaussian2
};

struct DftUnit
{
    int ctype{0};   // 4-bit ctype (D/B bit kept)
    int comp{0};
    bool is_db{false};
    int c1[3]{0, 0, 0}, c2[3]{0, 0, 0};       // closure corners, doubled coords
    int dim[3]{0, 0, 0};                      // closure dims
    bool has_local{false};
    int l1[3]{0, 0, 0};                       // local interior first corner, doubled
    int ldim[3]{0, 0, 0};                     // local dims (points)
    int i0[3]{0, 0, 0};                       // local box start in array indices
    std::vector<double> freqs;                // sorted, unique
    int64_t npoints() const { return has_local ? (int64_t)ldim[0] * ldim[1] * ldim[2] : 0; }
};

struct DftRequest
{
    int unit;
    std::vector<double> freqs;  // as requested (output order)
    std::string group;
};

struct GeomInfo
{
    std::string group;
    std::vector<double> x, y, z;
};

// Per-component material slots: the grid points whose medium differs from
// the default (dielectric or dispersive).  Everything else uses the default
// medium's coefficient.
struct SlotList
{
    std::vector<int64_t> lin;           // linear index
    std::vector<double> g;              // g_inf (epsilon for E, mu for H)
    std::vector<int> group;             // index into the side's pole groups
    std::vector<double> amp;            // [npole_stride][nslots], pole-major
    int npole_stride{0};
    bool any_poles{false};
};

struct PoleGroup
{
    std::vector<int> pool;  // pool indices of the active poles, increasing
};

struct Plan
{
    // Simulation::init scalars, src/simulation.cpp:133-141
    double courant{0.5}, resolution{1}, dx{1}, dt{0.5}, dx2{0.5};
    double sim_size[3]{0, 0, 0};
    int lo[3]{0, 0, 0}, hi[3]{0, 0, 0};  // doubled-coordinate range (sim_p1, sim_p2)
    int bc[3][2];
    // array layout
    int o[3]{0, 0, 0};
    int M[3]{0, 0, 0};
    int Mx_pad{0};
    int vlo[6][3], vhi[6][3];  // valid index range per component per axis
    bool precision_fp32{false};
    std::string engine{"auto"};
    // where the media are rasterised: "host" (build_plan / rasterize_media),
    // "device" (the engine's backend; an error if it cannot), "auto" (the
    // backend if it can, else the host)
    std::string rasterize{"auto"};
    int64_t divergence_check{4096};  // steps between checks for non-finite fields (0: never)
    uint64_t fused_wait_ns{2000000000ull};
    bool fused_stall_test{false};
    // CPML tables per axis and parity over array index (length M[a])
    std::vector<double> pml_k[3][2], pml_b[3][2], pml_c[3][2];
    bool any_pml{false};
    // media
    PoolMedium default_medium;
    double g_default[2]{1, 1};
    std::vector<Susceptibility> pool[2];
    std::vector<std::array<double, 3>> pool_coef[2];  // d1,d2,c3 per pool entry (increment form)
    std::vector<PoleGroup> groups[2];
    std::map<std::vector<int>, int> group_index[2];
    std::vector<Geometry> geoms;
    SlotList slots[6];
    // sources, in the reference's insertion order, split by side
    std::vector<Dipole> dipoles[2];
    double turnoff_time{0};
    Json sources_cfg;  // the config's "sources" array (replayed by rebuild_sources)
    bool has_sources{false};
    std::map<std::string, std::vector<double>> source_data;  // datasets the inhomogeneous sources read
    // DFT
    std::vector<DftUnit> units;
    std::vector<DftRequest> requests;
    std::vector<GeomInfo> geom_info;
    Json stop;
    bool has_stop{false};

    int64_t nx_total() const { return (int64_t)Mx_pad; }
    int64_t plane() const { return (int64_t)Mx_pad * M[1]; }
    int64_t cells() const { return (int64_t)Mx_pad * M[1] * M[2]; }
    int64_t lin(int i, int j, int k) const { return (int64_t)i + (int64_t)Mx_pad * ((int64_t)j + (int64_t)M[1] * k); }
    // first array index that can hold a grid point along axis a (kXFirst
    // along x, 1 along y and z; the indices before it are zero ghosts)
    static int first_index(int a) { return a == 0 ? kXFirst : 1; }
    int index_of(int a, int c) const { return ((c - o[a]) >> 1) + first_index(a); }
    int coord_of(int a, int i, int parity) const { return o[a] + 2 * (i - first_index(a)) + parity; }
    bool valid(int c, int i, int j, int k) const
    {
        return i >= vlo[c][0] && i <= vhi[c][0] && j >= vlo[c][1] && j <= vhi[c][1] && k >= vlo[c][2] && k <= vhi[c][2];
    }
    // Yee cell count used for throughput figures: (size/dx) per axis
    int64_t yee_cells() const;
};

struct Dataset
{
    const double *data{nullptr};
    uint64_t n{0};
};

// Builds the plan.  Throws std::runtime_error with a message on bad input.
void build_plan(const Json &cfg, const std::map<std::string, Dataset> &datasets, Plan &plan);

// Rebuilds the material slots (after a density dataset changed).
void rasterize_media(Plan &plan);

// Index box [r0, r1] (per axis) of component c's points that may lie inside
// geo: its bounding box with one point of margin, clipped to the component's
// valid range; false if empty.
bool geometry_index_range(const Plan &p, const Geometry &geo, int c, int r0[3], int r1[3]);

// Rebuilds the dipole lists from sources_cfg and source_data (after an
// inhomogeneous source's amplitude/phase datasets changed).
void rebuild_sources(Plan &plan);

// Component closure of a box (include/utility.hpp:546-552)
void component_closure(const double p1[3], const double p2[3], int ctype, int c1[3], int c2[3]);
} // namespace ffipg
