// C ABI (include/ffip_gb300.h) over the engine and the CUDA backend.
#include "../../include/ffip_gb300.h"
#include "../../include/ffip_gb300_surrogate.h"

#include <cstring>
#include <algorithm>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>

#include "engine.hpp"

namespace ffipg
{
Backend *new_default_backend(int device);  // the CUDA backend (kernels.cu); -1 = current device
void *backend_stream(Backend *be);
int adjoint_transpose(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz,
                      const double *pt, uint64_t npts, double *out);
int adjoint_sensitivity(double w_re, double w_im, double norm_re, double norm_im, const double *fwd, const double *adj,
                        const double *deps, const double *xyz, uint64_t n, const double *gx, uint64_t nx,
                        const double *gy, uint64_t ny, const double *gz, uint64_t nz, double *out);
int adjoint_transpose_noalloc(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz,
                              const double *pt, uint64_t npts, double *out);
uint64_t adjoint_transpose_noalloc_capacity();
int to_convolve(const double *in1, int n0, int n1, const double *in2, int m0, int m1, double *out, int transpose);
int check_inside(const double *req, uint64_t n, const double *poly, uint64_t m, unsigned char *out);
int sg_gemm(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs, float *C,
            int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream, int path);
int sg_check();
int sg_im2col(const void *x, const int *shape, const int *kernel, const int *stride, const int *pad, void *cols, void *stream);
int sg_col2im(const float *dcols, const int *shape, const int *kernel, const int *stride, const int *pad, float *dx, void *stream);
int sg_im2col_t(const void *x, const int *shape, const int *kernel, const int *stride, const int *pad, void *colsT, void *stream);
} // namespace ffipg

struct ffip_sim
{
    std::unique_ptr<ffipg::Backend> be;
    std::unique_ptr<ffipg::EngineBase> eng;
    std::vector<ffipg::OutputGroup> outs;
};

namespace
{
thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

int code_for(const std::exception &e)
{
    std::string m = e.what();
    if (m.rfind("CUDA error", 0) == 0 || m.find("no CUDA device") != std::string::npos) return FFIP_ERR_CUDA;
    return FFIP_ERR_INVALID;
}

template <typename F>
int guard(F &&f)
{
    try
    {
        return f();
    }
    catch (const std::bad_alloc &)
    {
        return fail(FFIP_ERR_INTERNAL, "host out of memory");
    }
    catch (const ffipg::Diverged &e)
    {
        return fail(FFIP_ERR_DIVERGED, e.what());
    }
    catch (const ffipg::DeviceTimeout &e)
    {
        return fail(FFIP_ERR_CUDA, e.what());
    }
    catch (const std::exception &e)
    {
        return fail(code_for(e), e.what());
    }
    catch (...)
    {
        return fail(FFIP_ERR_INTERNAL, "unknown error");
    }
}
} // namespace

extern "C" {

int ffip_create(const char *config_json, const ffip_dataset *datasets, uint64_t n_datasets, ffip_sim **out)
{
    return guard([&]() -> int {
        if (!config_json || !out) return fail(FFIP_ERR_INVALID, "ffip_create: null argument");
        *out = nullptr;
        ffipg::Json cfg = ffipg::Json::parse(config_json);
        std::map<std::string, ffipg::Dataset> ds;
        for (uint64_t i = 0; i < n_datasets; ++i)
        {
            if (!datasets[i].name || (!datasets[i].data && datasets[i].n)) return fail(FFIP_ERR_INVALID, "ffip_create: bad dataset entry");
            ds[datasets[i].name] = ffipg::Dataset{datasets[i].data, datasets[i].n};
        }
        ffipg::Plan plan;
        ffipg::build_plan(cfg, ds, plan);
        std::unique_ptr<ffip_sim> s(new ffip_sim);
        s->be.reset(ffipg::new_default_backend(cfg.has("device") ? cfg.at("device").integer() : -1));
        s->eng = ffipg::make_engine(std::move(plan), s->be.get());
        *out = s.release();
        return FFIP_OK;
    });
}

int ffip_step(ffip_sim *sim, int64_t n)
{
    return guard([&]() -> int {
        if (!sim) return fail(FFIP_ERR_INVALID, "null handle");
        if (n < 0) return fail(FFIP_ERR_INVALID, "negative step count");
        sim->eng->step(n);
        return FFIP_OK;
    });
}

int ffip_step_timed(ffip_sim *sim, int64_t n, double *ms)
{
    return guard([&]() -> int {
        if (!sim || !ms) return fail(FFIP_ERR_INVALID, "null argument");
        if (n < 0) return fail(FFIP_ERR_INVALID, "negative step count");
        *ms = sim->be->timed([&]() { sim->eng->step(n); });
        return FFIP_OK;
    });
}

int ffip_step_timed_pass(ffip_sim *sim, int64_t n, double *ms, double *pass_ms)
{
    return guard([&]() -> int {
        if (!sim || !ms || !pass_ms) return fail(FFIP_ERR_INVALID, "null argument");
        if (n < 0) return fail(FFIP_ERR_INVALID, "negative step count");
        sim->be->pass_ms();  // drop passes timed earlier
        sim->be->time_passes(true);
        try
        {
            *ms = sim->be->timed([&]() { sim->eng->step(n); });
        }
        catch (...)
        {
            sim->be->time_passes(false);
            throw;
        }
        sim->be->time_passes(false);
        *pass_ms = sim->be->pass_ms();
        return FFIP_OK;
    });
}

int ffip_run(ffip_sim *sim, const char *stop_json)
{
    return guard([&]() -> int {
        if (!sim) return fail(FFIP_ERR_INVALID, "null handle");
        if (stop_json)
        {
            ffipg::Json stop = ffipg::Json::parse(stop_json);
            sim->eng->run(stop);
        }
        else
        {
            if (!sim->eng->plan().has_stop) return fail(FFIP_ERR_INVALID, "config has no \"stop condition\"");
            sim->eng->run(sim->eng->plan().stop);
        }
        return FFIP_OK;
    });
}

int ffip_output_count(ffip_sim *sim, int *n)
{
    return guard([&]() -> int {
        if (!sim || !n) return fail(FFIP_ERR_INVALID, "null argument");
        sim->outs = sim->eng->outputs();
        *n = (int)sim->outs.size();
        return FFIP_OK;
    });
}

int ffip_output_group(ffip_sim *sim, int g, char *name, uint64_t cap)
{
    return guard([&]() -> int {
        if (!sim || !name || cap == 0) return fail(FFIP_ERR_INVALID, "null argument");
        if (g < 0 || g >= (int)sim->outs.size()) return fail(FFIP_ERR_NOT_FOUND, "output group index out of range (call ffip_output_count first)");
        const std::string &s = sim->outs[g].group;
        if (s.size() + 1 > cap) return fail(FFIP_ERR_INVALID, "name buffer too small");
        std::memcpy(name, s.c_str(), s.size() + 1);
        return FFIP_OK;
    });
}

int ffip_output_array(ffip_sim *sim, int g, const char *array, double *out, uint64_t n, uint64_t dims[4], int *ndim)
{
    return guard([&]() -> int {
        if (!sim || !array) return fail(FFIP_ERR_INVALID, "null argument");
        if (g < 0 || g >= (int)sim->outs.size()) return fail(FFIP_ERR_NOT_FOUND, "output group index out of range");
        const auto &G = sim->outs[g];
        for (size_t a = 0; a < G.names.size(); ++a)
        {
            if (G.names[a] != array) continue;
            if (ndim) *ndim = (int)G.shapes[a].size();
            if (dims)
                for (size_t d = 0; d < G.shapes[a].size() && d < 4; ++d) dims[d] = G.shapes[a][d];
            if (out)
            {
                if (n < G.data[a].size()) return fail(FFIP_ERR_INVALID, "output buffer too small");
                std::memcpy(out, G.data[a].data(), G.data[a].size() * sizeof(double));
            }
            return FFIP_OK;
        }
        return fail(FFIP_ERR_NOT_FOUND, std::string("no array '") + array + "' in group '" + G.group + "'");
    });
}

int ffip_set_density(ffip_sim *sim, const char *dataset, const double *rho, uint64_t n)
{
    return guard([&]() -> int {
        if (!sim || !dataset || (!rho && n)) return fail(FFIP_ERR_INVALID, "null argument");
        sim->eng->set_density(dataset, rho, n);
        return FFIP_OK;
    });
}

int ffip_set_source_data(ffip_sim *sim, const ffip_dataset *datasets, uint64_t n)
{
    return guard([&]() -> int {
        if (!sim || (!datasets && n)) return fail(FFIP_ERR_INVALID, "null argument");
        std::map<std::string, std::vector<double>> data;
        for (uint64_t i = 0; i < n; ++i)
        {
            if (!datasets[i].name || (!datasets[i].data && datasets[i].n)) return fail(FFIP_ERR_INVALID, "null dataset");
            data[datasets[i].name].assign(datasets[i].data, datasets[i].data + datasets[i].n);
        }
        sim->eng->set_source_data(data);
        return FFIP_OK;
    });
}

int ffip_reset(ffip_sim *sim)
{
    return guard([&]() -> int {
        if (!sim) return fail(FFIP_ERR_INVALID, "null handle");
        sim->eng->reset();
        return FFIP_OK;
    });
}

int ffip_get_stats(ffip_sim *sim, ffip_stats *st)
{
    return guard([&]() -> int {
        if (!sim || !st) return fail(FFIP_ERR_INVALID, "null argument");
        const ffipg::Plan &p = sim->eng->plan();
        st->time_step = sim->eng->time_step();
        st->yee_cells = p.yee_cells();
        st->array_cells = p.cells();
        st->dt = p.dt;
        st->dx = p.dx;
        st->bytes_per_step = sim->eng->bytes_per_step();
        st->pass_bytes_per_step = sim->eng->pass_bytes_per_step();
        st->kernel_launches = sim->eng->launches();
        st->fused = sim->eng->fused() ? 1 : 0;
        st->fp32 = p.precision_fp32 ? 1 : 0;
        st->h2d_bytes = sim->be->h2d_bytes;
        st->d2h_bytes = sim->be->d2h_bytes;
        return FFIP_OK;
    });
}

int ffip_sync(ffip_sim *sim)
{
    return guard([&]() -> int {
        if (!sim) return fail(FFIP_ERR_INVALID, "null handle");
        sim->be->sync();
        return FFIP_OK;
    });
}

void *ffip_stream(ffip_sim *sim) { return sim ? ffipg::backend_stream(sim->be.get()) : nullptr; }

int ffip_destroy(ffip_sim *sim)
{
    return guard([&]() -> int {
        if (!sim) return FFIP_OK;
        sim->eng.reset();
        sim->be.reset();
        delete sim;
        return FFIP_OK;
    });
}

const char *ffip_last_error(void) { return g_err.c_str(); }

int ffip_transpose(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz,
                   const double *pt, uint64_t npts, double *out)
{
    return guard([&]() -> int {
        if (!gx || !gy || !gz || !out || (!pt && npts)) return fail(FFIP_ERR_INVALID, "null argument");
        if (nx < 1 || ny < 1 || nz < 1) return fail(FFIP_ERR_INVALID, "some grid size is 0");
        return ffipg::adjoint_transpose(gx, nx, gy, ny, gz, nz, pt, npts, out);
    });
}

int ffip_sensitivity(double w_re, double w_im, double norm_re, double norm_im, const double *fwd, const double *adj, const double *deps,
                     const double *xyz, uint64_t n, const double *gx, uint64_t nx, const double *gy, uint64_t ny,
                     const double *gz, uint64_t nz, double *out)
{
    return guard([&]() -> int {
        if (!gx || !gy || !gz || !out || (n && (!fwd || !adj || !deps || !xyz))) return fail(FFIP_ERR_INVALID, "null argument");
        if (nx < 1 || ny < 1 || nz < 1) return fail(FFIP_ERR_INVALID, "some grid size is 0");
        return ffipg::adjoint_sensitivity(w_re, w_im, norm_re, norm_im, fwd, adj, deps, xyz, n, gx, nx, gy, ny, gz, nz, out);
    });
}

int ffip_to_convolve(const double *in1, uint64_t n0, uint64_t n1, const double *in2, uint64_t m0, uint64_t m1, double *out,
                     int transpose)
{
    return guard([&]() -> int {
        if (!out || (n0 && n1 && !in1) || !in2) return fail(FFIP_ERR_INVALID, "null argument");
        if (n0 > (1u << 30) || n1 > (1u << 30) || m0 > (1u << 30) || m1 > (1u << 30))
            return fail(FFIP_ERR_INVALID, "array too large");
        return ffipg::to_convolve(in1, (int)n0, (int)n1, in2, (int)m0, (int)m1, out, transpose);
    });
}

int ffip_check_inside(const double *req_pts, uint64_t n, const double *poly_pts, uint64_t m, uint8_t *out)
{
    return guard([&]() -> int {
        if ((n && (!req_pts || !out)) || (m && !poly_pts)) return fail(FFIP_ERR_INVALID, "null argument");
        if (n > (uint64_t(1) << 31) || m > (uint64_t(1) << 31)) return fail(FFIP_ERR_INVALID, "array too large");
        return ffipg::check_inside(req_pts, n, poly_pts, m, out);
    });
}

int ffip_flux(ffip_sim *sim, const char *e1_group, const char *h2_group, const double *x, uint64_t nx, const double *y,
              uint64_t ny, const double *z, uint64_t nz, const double *w, const double *freqs, uint64_t nf, double *flux)
{
    return guard([&]() -> int {
        if (!sim || !e1_group || !h2_group || !x || !y || !z || !w || !flux || (!freqs && nf))
            return fail(FFIP_ERR_INVALID, "null argument");
        if (!nx || !ny || !nz) return fail(FFIP_ERR_INVALID, "flux: empty integration grid");
        if (nx > (1u << 30) || ny > (1u << 30) || nz > (1u << 30) || nx * ny > (1ull << 40) || nx * ny * nz > (1ull << 40))
            return fail(FFIP_ERR_INVALID, "flux: integration grid too large");
        std::vector<double> vx(x, x + nx), vy(y, y + ny), vz(z, z + nz), vw(w, w + nx * ny * nz), vf(freqs, freqs + nf);
        auto r = sim->eng->flux(e1_group, h2_group, vx, vy, vz, vw, vf);
        std::copy(r.begin(), r.end(), flux);
        return FFIP_OK;
    });
}

int ffip_media_info(ffip_sim *sim, uint64_t checksum[6], int32_t *device)
{
    return guard([&]() -> int {
        if (!sim || !checksum || !device) return fail(FFIP_ERR_INVALID, "null argument");
        sim->eng->media_checksum(checksum);
        *device = sim->eng->device_media() ? 1 : 0;
        return FFIP_OK;
    });
}

int ffip_transpose_noalloc(const double *gx, uint64_t nx, const double *gy, uint64_t ny, const double *gz, uint64_t nz,
                           const double *pt, uint64_t npts, double *out)
{
    return guard([&]() -> int {
        if (!gx || !gy || !gz || !out || (!pt && npts)) return fail(FFIP_ERR_INVALID, "null argument");
        if (nx < 1 || ny < 1 || nz < 1) return fail(FFIP_ERR_INVALID, "some grid size is 0");
        const uint64_t cap = ffipg::adjoint_transpose_noalloc_capacity();
        if (nx > cap || ny > cap || nz > cap || nx * ny > cap || nx * ny * nz > cap)
            return fail(FFIP_ERR_INVALID, "ffip_transpose_noalloc: grid of " + std::to_string(nx) + " x " + std::to_string(ny) +
                                              " x " + std::to_string(nz) + " exceeds the fixed scratch of " +
                                              std::to_string(cap) + " doubles; use ffip_transpose");
        return ffipg::adjoint_transpose_noalloc(gx, nx, gy, ny, gz, nz, pt, npts, out);
    });
}

int ffip_sg_gemm(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs,
                 float *C, int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream)
{
    return guard([&]() -> int {
        if ((M > 0 && N > 0) && (!C || (K > 0 && (!A || !B)))) return fail(FFIP_ERR_INVALID, "null argument");
        return ffipg::sg_gemm(M, N, K, A, ars, acs, B, brs, bcs, C, crs, ccs, bias, accumulate, stream, 0);
    });
}

int ffip_sg_gemm_path(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs,
                      float *C, int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream, int path)
{
    return guard([&]() -> int {
        if ((M > 0 && N > 0) && (!C || (K > 0 && (!A || !B)))) return fail(FFIP_ERR_INVALID, "null argument");
        return ffipg::sg_gemm(M, N, K, A, ars, acs, B, brs, bcs, C, crs, ccs, bias, accumulate, stream, path);
    });
}

int ffip_sg_check(void)
{
    return guard([&]() -> int { return ffipg::sg_check(); });
}

int ffip_sg_im2col(const void *x, const int *shape5, const int *kernel3, const int *stride3, const int *pad3, void *cols,
                   void *stream)
{
    return guard([&]() -> int {
        if (!x || !shape5 || !kernel3 || !stride3 || !pad3 || !cols) return fail(FFIP_ERR_INVALID, "null argument");
        return ffipg::sg_im2col(x, shape5, kernel3, stride3, pad3, cols, stream);
    });
}

int ffip_sg_im2col_t(const void *x, const int *shape5, const int *kernel3, const int *stride3, const int *pad3, void *colsT,
                     void *stream)
{
    return guard([&]() -> int {
        if (!x || !shape5 || !kernel3 || !stride3 || !pad3 || !colsT) return fail(FFIP_ERR_INVALID, "null argument");
        return ffipg::sg_im2col_t(x, shape5, kernel3, stride3, pad3, colsT, stream);
    });
}

int ffip_sg_col2im(const float *dcols, const int *shape5, const int *kernel3, const int *stride3, const int *pad3, float *dx,
                   void *stream)
{
    return guard([&]() -> int {
        if (!dcols || !shape5 || !kernel3 || !stride3 || !pad3 || !dx) return fail(FFIP_ERR_INVALID, "null argument");
        return ffipg::sg_col2im(dcols, shape5, kernel3, stride3, pad3, dx, stream);
    });
}

} // extern "C"
