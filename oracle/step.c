/*
 * ORACLE — test infrastructure, not the product.
 *
 * Plain-C restatement of the reference's FDTD time-stepping loops, used as the
 * CPU oracle that the CUDA path is checked against, and as the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs load
 * it.  The data structures mirror the reference's on purpose so that results
 * match it bit for bit and its timing is representative:
 *
 *   - one interleaved doubled grid `eh` (E and H) and one `accdb`
 *     (running curl sum; D or B = accdb*dt), with a one-point ghost layer
 *     (include/fields.hpp:169-171, src/utility.cpp:130-140);
 *   - per-direction index lists for non-PML points (src/fields.cpp:133-148);
 *   - 72-byte array-of-structs PML points (include/fields.hpp:70-83,
 *     src/fields.cpp:89-109);
 *   - Gaussian dipole lists (src/fields.cpp:17-33);
 *   - constitutive/ADE groups keyed by susceptibility pattern
 *     (src/structure.cpp:56-85);
 *   - DFT units over component sub-boxes (src/dft.cpp:29-62);
 *   - the three ghost exchanges per half step (src/fields.cpp:327-482).
 *
 * The setup (JSON -> these arrays) is restated in numpy in oracle/port.py.
 * Loops over points are split across OpenMP threads; every point is written
 * by exactly one iteration, so the result does not depend on thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_PI 3.141592653589793e+00

/* src/fields.hpp:70-83 field order */
typedef struct {
    int64_t index;
    double phi1, b1, c1, inv_k1;
    double phi2, b2, c2, inv_k2;
} pml_point;

/* include/fields.hpp:33-40 */
typedef struct {
    int64_t index;
    double amp, start_time, end_time, width;
} dipole_point;

/* include/structure.hpp:346-350 */
typedef struct {
    int64_t index;
    double g_inf;
} medium_point;

typedef struct {
    int64_t npoints;
    int64_t npoles;
    const double *c1, *c2, *c3;   /* [npoles] */
    const medium_point *points;   /* [npoints] */
    const double *amp;            /* [npoints][npoles] */
    double *p, *p1;               /* [npoints][npoles] current and previous */
} medium_group;

typedef struct {
    int64_t npoints;
    int64_t is_db;
    int64_t nfreq;
    const int64_t *index;  /* [npoints] grid indices, x fastest */
    const double *freqs;   /* [nfreq] sorted */
    double *re, *im;       /* [nfreq][npoints] */
    double *buf;           /* [npoints] scratch */
} dft_unit;

typedef struct {
    double *eh, *accdb;
    int64_t size;
    int64_t strides[3];           /* +strides; H steps use the negation */
    double inv_dx, dt;
    pml_point *pml[2][3];         /* [0]=E side, [1]=H side */
    int64_t npml[2][3];
    const int64_t *curl[2][3];
    int64_t ncurl[2][3];
    const dipole_point *g1[2], *g2[2];
    int64_t ng1[2], ng2[2];
    double max_end[2];
    medium_group *groups[2];
    int64_t ngroups[2];
    dft_unit *dft[2];
    int64_t ndft[2];
    int64_t bc[3][2];             /* 0 PEC, 1 PMC, 2 None, 3 Sync, 4 Period */
    int64_t grid_p1[3], grid_p2[3], ghost_p1[3], dim[3];
    double *face_buf;             /* scratch for one face, 4 buffers */
    int64_t face_cap;
    int64_t time_step;
    int64_t nthreads;
} oracle_sim;

enum { BC_PEC = 0, BC_PMC = 1, BC_NONE = 2, BC_SYNC = 3, BC_PERIOD = 4 };

/* src/utility.cpp:260-272 */
static double gaussian1(double t, double width)
{
    double arg = (t / width);
    return arg * exp(-arg * arg / 2);
}

static double gaussian2(double t, double width)
{
    double arg = (t / width);
    arg = arg * arg;
    return (1 - arg) * exp(-arg);
}

/* PML_Stepping::step, src/fields.cpp:89-109 */
static void pml_step(oracle_sim *s, int side)
{
    const double *eh = s->eh;
    double *accdb = s->accdb;
    const double inv_dx = s->inv_dx;
    const int64_t sign = side == 0 ? 1 : -1;
    for (int i = 0; i < 3; ++i) {
        const int64_t stride1 = sign * s->strides[(i + 1) % 3];
        const int64_t stride2 = sign * s->strides[(i + 2) % 3];
        pml_point *pts = s->pml[side][i];
        const int64_t n = s->npml[side][i];
#pragma omp parallel for schedule(static) num_threads(s->nthreads)
        for (int64_t q = 0; q < n; ++q) {
            pml_point *pt = &pts[q];
            double curl1 = (eh[pt->index + stride1] - eh[pt->index - stride1]) * inv_dx;
            double curl2 = (eh[pt->index + stride2] - eh[pt->index - stride2]) * inv_dx;
            pt->phi1 = pt->b1 * pt->phi1 + pt->c1 * curl1;
            pt->phi2 = pt->b2 * pt->phi2 + pt->c2 * curl2;
            accdb[pt->index] += pt->phi1 - pt->phi2 + curl1 * pt->inv_k1 - curl2 * pt->inv_k2;
        }
    }
}

/* Curl_Stepping::step, src/fields.cpp:133-148 */
static void curl_step(oracle_sim *s, int side)
{
    const double *eh = s->eh;
    double *accdb = s->accdb;
    const double inv_dx = s->inv_dx;
    const int64_t sign = side == 0 ? 1 : -1;
    for (int i = 0; i < 3; ++i) {
        const int64_t stride1 = sign * s->strides[(i + 1) % 3];
        const int64_t stride2 = sign * s->strides[(i + 2) % 3];
        const int64_t *pts = s->curl[side][i];
        const int64_t n = s->ncurl[side][i];
#pragma omp parallel for schedule(static) num_threads(s->nthreads)
        for (int64_t q = 0; q < n; ++q) {
            int64_t p = pts[q];
            double curl1 = (eh[p + stride1] - eh[p - stride1]) * inv_dx;
            double curl2 = (eh[p + stride2] - eh[p - stride2]) * inv_dx;
            accdb[p] += (curl1 - curl2);
        }
    }
}

/* Gaussian_Dipoles_Stepping::step, src/fields.cpp:17-33 (sequential: several
 * dipoles may share one grid point and the order of the sums matters) */
static void dipole_step(oracle_sim *s, int side, double time)
{
    if (time > s->max_end[side]) return;
    double *accdb = s->accdb;
    for (int64_t q = 0; q < s->ng1[side]; ++q) {
        const dipole_point *p = &s->g1[side][q];
        if (time > p->start_time && time < p->end_time)
            accdb[p->index] += p->amp * gaussian1(time - (p->start_time + p->end_time) / 2, p->width);
    }
    for (int64_t q = 0; q < s->ng2[side]; ++q) {
        const dipole_point *p = &s->g2[side][q];
        if (time > p->start_time && time < p->end_time)
            accdb[p->index] += p->amp * gaussian2(time - (p->start_time + p->end_time) / 2, p->width);
    }
}

/* Medium_Stepping::step, src/structure.cpp:56-85 */
static void medium_step(oracle_sim *s, int side)
{
    double *eh = s->eh;
    const double *accdb = s->accdb;
    const double dt = s->dt;
    for (int64_t g = 0; g < s->ngroups[side]; ++g) {
        medium_group *grp = &s->groups[side][g];
        const int64_t stride = grp->npoles;
#pragma omp parallel for schedule(static) num_threads(s->nthreads)
        for (int64_t i = 0; i < grp->npoints; ++i) {
            int64_t index = grp->points[i].index;
            double g_inf = grp->points[i].g_inf;
            double *p = &grp->p[i * stride];
            double *p1 = &grp->p1[i * stride];
            const double *amp = &grp->amp[i * stride];
            double sum = 0.0;
            for (int64_t n = 0; n < stride; ++n) {
                double tmp = p[n];
                p[n] = grp->c1[n] * p[n] + grp->c2[n] * p1[n] + amp[n] * grp->c3[n] * eh[index];
                p1[n] = tmp;
            }
            for (int64_t n = 0; n < stride; ++n) sum = sum + p[n];   /* std::accumulate order */
            eh[index] = (accdb[index] * dt - sum) / g_inf;
        }
    }
}

static int64_t grid_index(const oracle_sim *s, int64_t x, int64_t y, int64_t z)
{
    return (x - s->ghost_p1[0]) + (y - s->ghost_p1[1]) * s->dim[0] + (z - s->ghost_p1[2]) * s->dim[0] * s->dim[1];
}

/* Iterates one face (all point types, stride 1, x fastest) at coordinate
 * `plane` along `dir`, over the interior extent in the other two directions;
 * copies eh values into buf (load=1) or buf into eh (load=0).
 * src/fields.cpp:433-463 */
static int64_t face_copy(oracle_sim *s, int dir, int64_t plane, double *buf, int load)
{
    int64_t lo[3], hi[3];
    for (int d = 0; d < 3; ++d) { lo[d] = s->grid_p1[d]; hi[d] = s->grid_p2[d]; }
    lo[dir] = hi[dir] = plane;
    int64_t n = 0;
    for (int64_t z = lo[2]; z <= hi[2]; ++z)
        for (int64_t y = lo[1]; y <= hi[1]; ++y)
            for (int64_t x = lo[0]; x <= hi[0]; ++x, ++n) {
                int64_t idx = grid_index(s, x, y, z);
                if (load) buf[n] = s->eh[idx];
                else s->eh[idx] = buf[n];
            }
    return n;
}

/* Fields::sync_boundary for one rank, src/fields.cpp:327-426 and
 * extract_symmetry_face src/fields.cpp:465-482 */
static void sync_boundary(oracle_sim *s, int dir)
{
    int64_t neg_bc = s->bc[dir][0], pos_bc = s->bc[dir][1];
    if (neg_bc == BC_NONE && pos_bc == BC_NONE) return;
    double *neg_send = s->face_buf, *pos_send = s->face_buf + s->face_cap;
    double *neg_recv = s->face_buf + 2 * s->face_cap, *pos_recv = s->face_buf + 3 * s->face_cap;
    int64_t n = 0;
    /* extraction */
    for (int side = 0; side < 2; ++side) {
        int64_t bc = side == 0 ? neg_bc : pos_bc;
        double *buf = side == 0 ? neg_send : pos_send;
        int64_t inner = side == 0 ? s->grid_p1[dir] + 1 : s->grid_p2[dir] - 1;
        if (bc == BC_PEC || bc == BC_PMC) {
            int64_t phase = bc == BC_PEC ? -1 : 1;
            int64_t pos = side == 0 ? s->grid_p1[dir] : s->grid_p2[dir];
            int64_t mult = (pos & 1) ? phase : -phase;
            n = face_copy(s, dir, inner, buf, 1);
            for (int64_t i = 0; i < n; ++i) buf[i] *= mult;
        } else if (bc == BC_PERIOD) {
            n = face_copy(s, dir, inner, buf, 1);
        }
    }
    /* single-rank exchange: periodic neighbours are this rank */
    if (pos_bc == BC_PERIOD) memcpy(neg_recv, pos_send, (size_t)n * sizeof(double));
    if (neg_bc == BC_PERIOD) memcpy(pos_recv, neg_send, (size_t)n * sizeof(double));
    /* assignment */
    for (int side = 0; side < 2; ++side) {
        int64_t bc = side == 0 ? neg_bc : pos_bc;
        int64_t ghost = side == 0 ? s->grid_p1[dir] - 1 : s->grid_p2[dir] + 1;
        if (bc == BC_PEC || bc == BC_PMC)
            face_copy(s, dir, ghost, side == 0 ? neg_send : pos_send, 0);
        else if (bc == BC_PERIOD)
            face_copy(s, dir, ghost, side == 0 ? neg_recv : pos_recv, 0);
    }
}

/* DFT_Unit::update, src/dft.cpp:29-62 */
static void dft_step(oracle_sim *s, int side, double time)
{
    for (int64_t u = 0; u < s->ndft[side]; ++u) {
        dft_unit *d = &s->dft[side][u];
        const int64_t n = d->npoints;
        if (n == 0) continue;
        for (int64_t i = 0; i < n; ++i)
            d->buf[i] = d->is_db ? s->accdb[d->index[i]] * s->dt : s->eh[d->index[i]];
        for (int64_t f = 0; f < d->nfreq; ++f) {
            double cos_wt = cos(2 * ORACLE_PI * d->freqs[f] * time);
            double sin_wt = -sin(2 * ORACLE_PI * d->freqs[f] * time);
            double *re = d->re + f * n, *im = d->im + f * n;
#pragma omp parallel for schedule(static) num_threads(s->nthreads)
            for (int64_t i = 0; i < n; ++i) {
                im[i] += sin_wt * d->buf[i];
                re[i] += cos_wt * d->buf[i];
            }
        }
    }
}

/* Simulation::step_m / step_e, src/simulation.cpp:748-766 */
static void half_step(oracle_sim *s, int side)
{
    double src_time = side == 1 ? s->time_step * s->dt : (s->time_step + 0.5) * s->dt;
    double dft_time = side == 1 ? (s->time_step + 0.5) * s->dt : (s->time_step + 1) * s->dt;
    pml_step(s, side);
    curl_step(s, side);
    dipole_step(s, side, src_time);
    medium_step(s, side);
    for (int d = 0; d < 3; ++d) sync_boundary(s, d);
    dft_step(s, side, dft_time);
}

/* One loop iteration of Simulation::run_until_time, src/simulation.cpp:773-779 */
int oracle_run_steps(oracle_sim *s, int64_t nsteps)
{
    if (s->nthreads < 1) s->nthreads = 1;
    for (int64_t i = 0; i < nsteps; ++i) {
        half_step(s, 1);
        half_step(s, 0);
        s->time_step += 1;
    }
    return 0;
}

int oracle_struct_size(void) { return (int)sizeof(oracle_sim); }
