/*
 * ffip_gb300 — C ABI of the GB300 (sm_103a) FDTD stepper.
 *
 * The reference (ffip) has no C ABI: its hot path is reached through the
 * run_sim_json CLI (app/run_sim_json.cpp:6-25), which reads config.json and
 * the HDF5 input file, runs Simulation::init / run / output
 * (src/simulation.cpp:127-188, 903-958, 967-977) and writes the HDF5 output
 * file, and through the pybind module _ffip (app/ffip.cpp:390-415).  Each
 * entry point below names the reference interface it replaces.  The config
 * JSON is the reference's schema unchanged (what ffip/simulation.py:362-402
 * emits); input datasets are passed as named float64 arrays instead of an
 * HDF5 file; outputs are read back as named float64 arrays with the
 * reference's dataset names and shapes.
 *
 * Conventions: every function returns 0 (FFIP_OK) or a negative error code
 * and never aborts; ffip_last_error() gives the message of the calling
 * thread's last failure.  Host buffers belong to the caller; device memory
 * belongs to the handle.  Calls on one handle must be serialised; distinct
 * handles hold separate state (fields, streams, job lists), but driving
 * several handles from several host threads at once is not supported: call
 * them from one thread.  A handle runs on one CUDA device, on its own
 * streams.
 */
#ifndef FFIP_GB300_H
#define FFIP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFIP_OK 0
#define FFIP_ERR_INVALID (-1)   /* bad argument, config or dataset */
#define FFIP_ERR_CUDA (-2)      /* CUDA runtime failure (no device, out of memory, ...) */
#define FFIP_ERR_NOT_FOUND (-3) /* unknown output group / array / dataset */
#define FFIP_ERR_INTERNAL (-4)
#define FFIP_ERR_DIVERGED (-5)  /* the divergence check found NaN / infinite field values */

typedef struct ffip_sim ffip_sim;

/* One named input dataset (the reference reads these from "input file",
 * src/simulation.cpp:151-153,301-306,431-496; ffip/geom.py:432-433,528-545;
 * ffip/source.py:127-129). Arrays are flattened in [z][y][x] order. */
typedef struct ffip_dataset {
    const char *name;
    const double *data;
    uint64_t n;
} ffip_dataset;

typedef struct ffip_stats {
    int64_t time_step;       /* completed time steps */
    int64_t yee_cells;       /* (size/dx) per axis, multiplied */
    int64_t array_cells;     /* padded cells per component array */
    double dt, dx;
    double bytes_per_step;   /* algorithmic bytes of one time step */
    int64_t kernel_launches; /* kernel launches issued so far */
    int32_t fused;           /* 1 = fused H+E pass, 0 = separate H and E passes */
    int32_t fp32;            /* 1 = fp32 field state, 0 = fp64 */
    uint64_t h2d_bytes;      /* host->device bytes copied so far */
    uint64_t d2h_bytes;      /* device->host bytes copied so far */
    double pass_bytes_per_step; /* bytes_per_step without the DFT sums: the field pass's share */
} ffip_stats;

/* Simulation::init(config) (src/simulation.cpp:127-188): parses the config
 * JSON, builds the grid, CPML, media, sources and DFT monitors, and uploads
 * them to a CUDA device.  Rebuild-only keys: "precision" ("fp64" default,
 * "fp32" = fp32 field state with fp64 DFT sums), "engine" ("auto" and
 * "fused": the fused pass; "unfused": separate H and E passes), "device"
 * (CUDA device index; default: the device current in the calling thread),
 * "divergence check interval" (every that many steps the fields are checked
 * for NaN / infinite values and stepping stops with FFIP_ERR_DIVERGED;
 * default 4096, 0 = never; the reference has no such check), "fused wait
 * timeout" (seconds after which a wait inside the fused pass gives up; the
 * next synchronising call then returns FFIP_ERR_CUDA and the fields stay
 * invalid until ffip_reset; default 2) and "fused wait test" (true: every CTA
 * of the fused pass first waits on a barrier that nothing completes, so that
 * the timeout path can be tested). */
int ffip_create(const char *config_json, const ffip_dataset *datasets, uint64_t n_datasets, ffip_sim **out);

/* n iterations of the time loop body of Simulation::run_until_time
 * (step_m, step_e, ++time_step; src/simulation.cpp:773-779). */
int ffip_step(ffip_sim *sim, int64_t n_steps);

/* ffip_step with device timing: CUDA events recorded on the handle's stream
 * before and after the n steps; *ms receives the elapsed device time.
 * Blocks until the steps have finished. */
int ffip_step_timed(ffip_sim *sim, int64_t n_steps, double *ms);

/* ffip_step_timed that also times the field pass of every step: CUDA events
 * on the handle's stream from the launch of the first k_fused instance to
 * the point where both instances (and the face-layer kernels that run beside
 * them) have finished, summed over the n steps into *pass_ms.  *pass_ms is 0
 * for the separate H and E passes ("engine": "unfused").  Every 1024 passes
 * the host waits for the passes issued so far (the events are reused). */
int ffip_step_timed_pass(ffip_sim *sim, int64_t n_steps, double *ms, double *pass_ms);

/* Simulation::run(stop_cond) (src/simulation.cpp:903-958): "time", "decay"
 * or DFT steady-state stop conditions.  stop_json == NULL uses the config's
 * "stop condition".  Like the reference, time_step restarts from 0 only at
 * creation / ffip_reset. */
int ffip_run(ffip_sim *sim, const char *stop_json);

/* Output datasets, as Simulation::output writes them (src/simulation.cpp:
 * 967-977, src/dft.cpp:273-320, geometry info src/simulation.cpp:190-233).
 * ffip_output_count collects the current values from the device. */
int ffip_output_count(ffip_sim *sim, int *n_groups);
int ffip_output_group(ffip_sim *sim, int group, char *name, uint64_t name_cap);
/* Copies array `array` ("real", "imag", "x", "y", "z", "f") of group `group`
 * into out[n] (out may be NULL to query the shape); dims/ndim receive the
 * shape ([nf, nz, ny, nx] for real/imag). */
int ffip_output_array(ffip_sim *sim, int group, const char *array, double *out, uint64_t n, uint64_t dims[4], int *ndim);

/* Replaces the density of the two-medium / general medium boxes that read
 * `dataset` (src/simulation.cpp:423-439; Two_Medium_Box, src/geometry.cpp:
 * 49-76), re-derives the media and resets the fields to time step 0 — one
 * design iteration without re-parsing the config. */
int ffip_set_density(ffip_sim *sim, const char *dataset, const double *rho, uint64_t n);

/* Replaces amplitude / phase datasets of the inhomogeneous sources that read
 * them (Simulation::set_inhom_source, src/simulation.cpp:284-336; written by
 * Inhom_Source.dump, ffip/source.py:126-129 — the adjoint sources of
 * Adjoint_Source.eval_functionals_and_set_sources, ffip/simulation.py:
 * 728-753), rebuilds the dipoles and resets the fields to time step 0 — the
 * adjoint run of a design iteration without re-parsing the config.  Each
 * dataset must keep its size; a name no inhomogeneous source reads is an
 * error (FFIP_ERR_INVALID). */
int ffip_set_source_data(ffip_sim *sim, const ffip_dataset *datasets, uint64_t n);

/* Zeroes fields, auxiliary state and DFT sums; time_step = 0. */
int ffip_reset(ffip_sim *sim);

int ffip_get_stats(ffip_sim *sim, ffip_stats *stats);

/* Flux_Region.get_values (ffip/simulation.py:121-160) on the device: the
 * Poynting flux, the sum over the integration points of Re(E1 conj(H2))
 * times the point's weight, per frequency, where E1 / H2 are the DFT monitor
 * groups e1_group / h2_group (output group names) interpolated linearly over
 * their output grids (the reference's Fields_DFT interpolant,
 * ffip/simulation.py:55-91).  The points are the grid x[nx] x y[ny] x z[nz];
 * w[nz][ny][nx] are their weights (the reference's get_int_weights); freqs
 * must be frequencies of both monitors (at most 64).  flux[nf] receives the
 * sums; the monitors stay on the device. */
int ffip_flux(ffip_sim *sim, const char *e1_group, const char *h2_group, const double *x, uint64_t nx, const double *y,
              uint64_t ny, const double *z, uint64_t nz, const double *w, const double *freqs, uint64_t nf, double *flux);

/* The handle's material tables: an FNV-1a hash per component of the slot
 * map, row ranges, g_inf, dt/g_inf, 1/g_inf, pole group, packed record and
 * pole amplitudes as they sit on the device (equal hashes: equal tables),
 * and *device = 1 when the media were rasterised on the GPU (config key
 * "rasterize": "auto" (default: on the GPU where the geometry allows),
 * "device" or "host"; ffip_set_density rasterises again where the handle
 * did first).  The rasterisation follows Structure::set_materials_from_
 * geometry and the density boxes' get_medium (src/structure.cpp:155-249,
 * src/geometry.cpp:49-107); no reference interface reads the tables back. */
int ffip_media_info(ffip_sim *sim, uint64_t checksum[6], int32_t *device);

/* Blocks until all work of the handle has finished. */
int ffip_sync(ffip_sim *sim);

/* The handle's cudaStream_t, for callers that order their own work with it. */
void *ffip_stream(ffip_sim *sim);

int ffip_destroy(ffip_sim *sim);

const char *ffip_last_error(void);

/* _ffip.transpose (app/ffip.cpp:308-352): adjoint of trilinear interpolation
 * with zero-padded extrapolation (include/utility.hpp:706-749).  Scatter-adds
 * pt[i][3] at (pt[i][0], pt[i][1], pt[i][2]) onto the grid gx[nx] x gy[ny] x
 * gz[nz] (uniform spacing from the first two entries); out[nz][ny][nx] is
 * overwritten.  Host buffers; runs on the current CUDA device. */
int ffip_transpose(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz,
                   const double *pt, uint64_t npts, double *out);

/* Adjoint_Volume.get_sensitivity (ffip/simulation.py:841-869) on the device:
 * for each of n points, se = Re(w * fwd * adj * deps / norm) with complex fwd,
 * adj and deps (d epsilon / d rho) given as interleaved (re, im) pairs, then
 * the transpose of trilinear interpolation of se onto the density grid, as
 * ffip_transpose.  w = 2 pi j f reproduces the reference's formula;
 * w = 2 j sin(pi f dt) / dt is the exact factor of the leap-frog E update.
 * Points are (x, y, z) triples.  out[nz][ny][nx] is overwritten. */
int ffip_sensitivity(double w_re, double w_im, double norm_re, double norm_im, const double *fwd, const double *adj,
                     const double *deps, const double *xyz, uint64_t n, const double *gx, uint64_t nx,
                     const double *gy, uint64_t ny, const double *gz, uint64_t nz, double *out);

/* _ffip.TO_convolve / _ffip.TO_convolve_transpose (app/ffip.cpp:222-306):
 * the density filter of the design scripts.  transpose = 0: out[i][j] is the
 * average of in1 over the in-bounds part of the filter window centred at
 * (i, j), weighted by the filter in2[m0][m1] (odd sizes); transpose = 1: its
 * transpose.  in1 and out are n0 x n1, row-major, host buffers.  As in the
 * reference, both filter axes are indexed with the first half-width, so only
 * filters with equal half-widths are accepted. */
int ffip_to_convolve(const double *in1, uint64_t n0, uint64_t n1, const double *in2, uint64_t m0, uint64_t m1, double *out,
                     int transpose);

/* _ffip.check_inside (app/ffip.cpp:353-387): out[i] = 1 when query point i,
 * (req_pts[2i], req_pts[2i+1]), lies strictly inside the polygon of m
 * vertices (poly_pts[2j], poly_pts[2j+1]) -- CGAL's Polygon_2::bounded_side
 * == ON_BOUNDED_SIDE -- and 0 on an edge, on a vertex or outside.  The polygon
 * is simple; its first vertex may be repeated at the end (a closed ring).
 * Orientation tests are exact.  At most 2^31 points and 2^31 vertices.  Host
 * buffers; computed on the current CUDA device. */
int ffip_check_inside(const double *req_pts, uint64_t n, const double *poly_pts, uint64_t m, uint8_t *out);

/* ffip_transpose without any device allocation.  No counterpart in the
 * reference (its transpose runs on the host).  Same arguments, result and
 * errors as ffip_transpose, but the points and the output grid are staged in
 * one fixed 8 MiB device buffer compiled into the library (a file-scope
 * __device__ array) instead of cudaMalloc/cudaFree per call.  For callers
 * that must not allocate: a process whose HBM is fully committed to field
 * arrays, where a per-call cudaMalloc fails, and a density-update loop that
 * runs beside a stepping simulation, where cudaMalloc/cudaFree would
 * synchronise the device.
 * Limit: 4 * npts + nx * ny * nz <= 1048576 doubles; larger inputs return
 * FFIP_ERR_INVALID with a message, use ffip_transpose for them.
 * The output part of the buffer is zeroed by every call.  The buffer is
 * shared by all calls on a device: calls that overlap on one device (from
 * several threads) race and must be serialised by the caller.  Every call
 * looks the buffer's address up with cudaGetSymbolAddress on the current
 * device (nothing is cached between calls); the first call on a device
 * also loads the library's device code there, so make that first call
 * outside any stream capture. */
int ffip_transpose_noalloc(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz,
                           const double *pt, uint64_t npts, double *out);

#ifdef __cplusplus
}
#endif
#endif /* FFIP_GB300_H */
