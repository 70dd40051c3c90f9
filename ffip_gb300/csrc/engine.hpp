// Time-stepping engine: owns the device state of one simulation and drives
// the kernels in the reference's half-step order (Simulation::step_m /
// step_e, src/simulation.cpp:748-766).  Memory and launches go through a
// Backend; the product library links the CUDA backend (kernels.cu).
#pragma once
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "plan.hpp"
#include "stencil.cuh"

namespace ffipg
{
// Fused H+E pass parameters (None boundaries, no magnetic poles): the H
// update of one z plane and the E update of the same plane in one kernel,
// ping-ponging field buffers between steps.  See kernels.cu.
template <typename T>
struct FusedParams
{
    SideParams<T> h, e;   // h.f/e.f = output buffers, h.o/e.o unused
    const T *ein[3];      // E at step n (input buffers)
    const T *hin[3];      // H at step n-1/2 (input buffers)
    T *eout[3], *hout[3]; // outputs
    const T *psih_in[3][2];
    T *psih_out[3][2];
    // the pass's waits on its TMA rings and on the threads of its CTA give
    // up after wait_ns (global timer) and report a timeout; stall_test != 0
    // makes every CTA first wait on a barrier that nothing completes (the
    // timeout path, exercised by a test)
    uint64_t wait_ns;
    int stall_test;
};

// The PEC / PMC / periodic ghost faces of a plan (Fields::sync_boundary,
// src/fields.cpp:327-482); returns their number
int build_ghost_faces(const Plan &P, GhostFace *faces, int max_faces);

// A bounded wait inside a kernel gave up: the results of the steps since
// the last check are invalid.
struct DeviceTimeout : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

// The device rasterisation does not cover a geometry of the plan (the
// engine then rasterises on the host unless "device" was asked for).
struct RasterUnsupported : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

// The divergence check found non-finite field values.
struct Diverged : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

// Material tables of one component built on the device (Backend::rasterize):
// the arrays init_media uploads from a host SlotList, in device memory from
// the engine's allocator; g, coef, inv, rec and amp hold the field type
struct RasterComp
{
    int64_t n{0};         // slots
    int stride{0};        // most active poles of one slot
    int64_t pole_sum{0};  // active poles summed over the slots
    int *map{nullptr};
    RowRange *rows{nullptr};
    void *g{nullptr}, *coef{nullptr}, *inv{nullptr}, *rec{nullptr}, *amp{nullptr};
    uint8_t *group{nullptr};
};

struct Backend
{
    virtual ~Backend() {}
    virtual void *alloc(size_t bytes) = 0;  // returns zero-filled memory
    virtual void release(void *p) = 0;
    virtual void h2d(void *dst, const void *src, size_t bytes) = 0;
    virtual void d2h(void *dst, const void *src, size_t bytes) = 0;
    virtual void zero(void *p, size_t bytes) = 0;
    virtual void sync() = 0;
    virtual void update(const SideParams<double> &p, bool is_e) = 0;
    virtual void update(const SideParams<float> &p, bool is_e) = 0;
    virtual bool has_fused() const { return false; }
    // one fused time step; returns the number of kernels it launched.
    // hghost (may be null): the H ghost faces (PEC / PMC / periodic), filled
    // in the new H between the pass and the E points that read them
    virtual int fused(const FusedParams<double> &, const GhostParams<double> *) { return 0; }
    virtual int fused(const FusedParams<float> &, const GhostParams<float> *) { return 0; }
    virtual void sources(const SourceParams<double> &p) = 0;
    virtual void sources(const SourceParams<float> &p) = 0;
    virtual void ghosts(const GhostParams<double> &p) = 0;
    virtual void ghosts(const GhostParams<float> &p) = 0;
    // value of a trilinear probe (up to 8 weighted points) -> out[0]
    virtual void probe(const double *f, const int64_t *lin, const double *w, int n, double *out) = 0;
    virtual void probe(const float *f, const int64_t *lin, const double *w, int n, double *out) = 0;
    // sum over i of re[i]^2 + im[i]^2 -> out[0]
    virtual void dft_norm(const double *re, const double *im, int64_t n, double *out) = 0;
    // whether any of the first n values of any of the nf arrays is NaN or
    // infinite (waits for the result)
    virtual bool any_nonfinite(const double *const *f, int nf, int64_t n) = 0;
    virtual bool any_nonfinite(const float *const *f, int nf, int64_t n) = 0;
    // forgets a reported kernel timeout (after the state was reset)
    virtual void clear_error() {}
    // out[f] = sum over the integration points of flux_point(A, t, f); the
    // coordinate and weight arrays of A are host arrays, uploaded here
    virtual void flux(const FluxArgs &A, double *out) = 0;
    // rasterises the media of `plan` (geometry list, default medium,
    // susceptibility pools) on the device: the slot tables of the six
    // components (field type float when fp32) in memory from alloc, and the
    // pole groups of both sides numbered by first appearance, as
    // rasterize_media numbers them
    virtual bool can_rasterize() const { return false; }
    virtual void rasterize(const Plan &plan, bool fp32, const std::function<void *(size_t)> &alloc, RasterComp out[6],
                           std::vector<PoleGroup> groups[2])
    {
        (void)plan, (void)fp32, (void)alloc, (void)out, (void)groups;
        throw std::runtime_error("this backend does not rasterise media");
    }
    virtual const char *name() const = 0;
    // device time of f() between events on the backend's stream (ms)
    virtual double timed(const std::function<void()> &f) = 0;
    // while on, every fused pass is bracketed by timing events on the
    // backend's stream (from the launch of the first k_fused instance to the
    // point where both instances, and the face-layer kernels beside them,
    // have finished); pass_ms() waits for them and returns the summed
    // device time (ms) of the passes since the last call, 0 where the
    // backend does not time passes
    virtual void time_passes(bool on) { (void)on; }
    virtual double pass_ms() { return 0.0; }
    uint64_t h2d_bytes{0}, d2h_bytes{0};
};

struct OutputGroup
{
    std::string group;
    std::vector<std::string> names;
    std::vector<std::vector<uint64_t>> shapes;
    std::vector<std::vector<double>> data;
};

class EngineBase
{
public:
    virtual ~EngineBase() {}
    virtual void step(int64_t n) = 0;
    virtual void run(const Json &stop) = 0;
    virtual int64_t time_step() const = 0;
    virtual std::vector<OutputGroup> outputs() = 0;
    virtual void reset() = 0;
    virtual void set_density(const std::string &dataset, const double *rho, uint64_t n) = 0;
    // new amplitude/phase datasets of inhomogeneous sources; zeroes the state
    virtual void set_source_data(const std::map<std::string, std::vector<double>> &data) = 0;
    virtual const Plan &plan() const = 0;
    virtual bool fused() const = 0;
    virtual int64_t launches() const = 0;  // kernel launches issued so far
    // algorithmic bytes of one full time step, and the number of Yee cells
    virtual double bytes_per_step() const = 0;
    // bytes_per_step without the DFT sums (the field pass's share)
    virtual double pass_bytes_per_step() const = 0;
    // Poynting flux through a flux region per frequency from the E1 / H2
    // monitor groups (their names), the integration points and weights
    // FNV-1a hash of each component's device material tables (slot count,
    // pole stride, slot map, row ranges, g_inf, dt/g_inf, 1/g_inf, group,
    // packed record, amplitudes): equal hashes mean equal tables
    virtual void media_checksum(uint64_t out[6]) = 0;
    // whether the media were rasterised on the device
    virtual bool device_media() const = 0;
    virtual std::vector<double> flux(const std::string &e1_group, const std::string &h2_group, const std::vector<double> &x,
                                     const std::vector<double> &y, const std::vector<double> &z, const std::vector<double> &w,
                                     const std::vector<double> &freqs) = 0;
};

std::unique_ptr<EngineBase> make_engine(Plan &&plan, Backend *be);
} // namespace ffipg
