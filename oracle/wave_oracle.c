/*
 * wave_oracle.c -- CPU restatement of simwave's forward time loop.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the oracle for the GPU library.
 * It is built into oracle/_build/liboracle.so and is loaded only by tests/,
 * by __graft_entry__.smoke() and by bench.py's CPU-baseline leg. The product
 * (simwave_gb300) never links or calls it.
 *
 * It restates the reference C path (the numerical contract) section by
 * section, with the same arithmetic, operation order and float/double
 * promotions, so that a build with the reference's flags reproduces the
 * reference bit for bit:
 *   simwave/kernel/backend/c_code/forward/constant_density/2d/wave.c:23-559
 *   simwave/kernel/backend/c_code/forward/variable_density/2d/wave.c:23-585
 *   simwave/kernel/backend/c_code/forward/constant_density/3d/wave.c:23-663
 *   simwave/kernel/backend/c_code/forward/variable_density/3d/wave.c:23-691
 *
 * Build once per precision with -DREAL=float -DSFX=f32 or -DREAL=double
 * -DSFX=f64, and -std=c99 -ffp-contract=off so no FMA contraction changes
 * the rounding on either x86-64 or aarch64.
 *
 * Sections per time step n = begin..end (inclusive), as in the reference:
 *   1 stencil: u_next = 2/D u_cur - N/D u_prev + dt^2 v^2 L(u_cur) / D
 *   2 sources: u_next += dt^2 v^2 kws w[n-1] / D over each KWS window
 *   3 boundary conditions on u_next (none / null Dirichlet / null Neumann)
 *   4 receivers: rec[n-1] = sum kws u_cur over each KWS window
 *   5 slot bookkeeping for the saving stride (incl. the even-stride swap)
 */
#include <stddef.h>
#include <sys/time.h>

#ifndef REAL
#error "define REAL (float or double)"
#endif
#ifndef SFX
#error "define SFX (f32 or f64)"
#endif

typedef REAL real;

#define CAT_(a, b) a##_##b
#define CAT(a, b) CAT_(a, b)
#define EXPORT(name) CAT(name, SFX)

enum { BC_NONE = 0, BC_DIRICHLET = 1, BC_NEUMANN = 2 };

static double wall_seconds(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (double)tv.tv_sec + (double)tv.tv_usec / 1000000.0;
}

/* ---- time-level slot bookkeeping (wave.c:110-122 and 466-514) ---------- */

typedef struct {
    size_t prev, cur, next;
} slot_state;

/* Slots used by step n before its stencil runs. */
static void slots_at_step(slot_state *s, size_t n, size_t stride)
{
    if (stride == 0) {
        s->prev = (n - 1) % 3;
        s->cur = n % 3;
        s->next = (n + 1) % 3;
    } else if (stride == 1) {
        s->prev = n - 1;
        s->cur = n;
        s->next = n + 1;
    }
}

/* After step n: move to the next slot pair. Returns 1 when the reference
 * exchanges the contents of slots cur and next (even stride). */
static int slots_after_step(slot_state *s, size_t n, size_t stride, size_t last)
{
    if (stride <= 1)
        return 0;
    if (n % stride == 1) {
        s->prev = s->cur;
        s->cur += 1;
        s->next += 1;
        if (stride % 2 == 0 && n < last) {
            size_t t = s->cur;
            s->cur = s->next;
            s->next = t;
            return 1;
        }
        return 0;
    }
    s->prev = s->cur;
    s->cur = s->next;
    s->next = s->prev;
    return 0;
}

static void exchange_slots(real *a, real *b, size_t count)
{
    #pragma omp parallel for
    for (size_t i = 0; i < count; i++) {
        real t = a[i];
        a[i] = b[i];
        b[i] = t;
    }
}

/* ---- section 1: the damped leapfrog update of one point ----------------- */

/* Final update given the spatial operator `value` (already summed), the
 * reference's promotions: slowness and D/N are formed in double and rounded,
 * the last line is evaluated in double (wave.c:170-178). */
static inline real leapfrog(real value, real vel, real damp, real dt,
                            real dt2, real ucur, real uprev)
{
    real slowness = 1.0 / (vel * vel);
    real den = (1.0 + damp * dt / (2 * slowness));
    real num = (1.0 - damp * dt / (2 * slowness));
    value *= (dt2 / slowness) / den;
    return 2.0 / den * ucur - (num / den) * uprev + value;
}

static void stencil_2d_cd(real *restrict un, const real *restrict uc,
                          const real *restrict up, const real *vel,
                          const real *damp, const real *c2, size_t r,
                          size_t nz, size_t nx, real dz, real dx, real dt)
{
    real dz2 = dz * dz, dx2 = dx * dx, dt2 = dt * dt;
    #pragma omp parallel for
    for (size_t i = r; i < nz - r; i++) {
        for (size_t j = r; j < nx - r; j++) {
            size_t p = i * nx + j;
            real value = 0.0;
            real sx = c2[0] * uc[p];
            real sz = c2[0] * uc[p];
            for (size_t k = 1; k <= r; k++) {
                sx += c2[k] * (uc[p + k] + uc[p - k]);
                sz += c2[k] * (uc[p + k * nx] + uc[p - k * nx]);
            }
            value += sx / dx2 + sz / dz2;
            un[p] = leapfrog(value, vel[p], damp[p], dt, dt2, uc[p], up[p]);
        }
    }
}

static void stencil_2d_vd(real *restrict un, const real *restrict uc,
                          const real *restrict up, const real *vel,
                          const real *den, const real *damp, const real *c2,
                          const real *c1, size_t r, size_t nz, size_t nx,
                          real dz, real dx, real dt)
{
    real dz2 = dz * dz, dx2 = dx * dx, dt2 = dt * dt;
    #pragma omp parallel for
    for (size_t i = r; i < nz - r; i++) {
        for (size_t j = r; j < nx - r; j++) {
            size_t p = i * nx + j;
            real value = 0.0;
            real sdx = c2[0] * uc[p], sdz = c2[0] * uc[p];
            real fux = 0.0, fuz = 0.0, frx = 0.0, frz = 0.0;
            for (size_t k = 1; k <= r; k++) {
                sdx += c2[k] * (uc[p + k] + uc[p - k]);
                fux += c1[k] * (uc[p + k] - uc[p - k]);
                frx += c1[k] * (den[p + k] - den[p - k]);
                sdz += c2[k] * (uc[p + k * nx] + uc[p - k * nx]);
                fuz += c1[k] * (uc[p + k * nx] - uc[p - k * nx]);
                frz += c1[k] * (den[p + k * nx] - den[p - k * nx]);
            }
            value += sdx / dx2 + sdz / dz2;
            real tx = (fux * frx) / (4 * dx2);
            real tz = (fuz * frz) / (4 * dz2);
            value -= (tx + tz) / den[p];
            un[p] = leapfrog(value, vel[p], damp[p], dt, dt2, uc[p], up[p]);
        }
    }
}

static void stencil_3d_cd(real *restrict un, const real *restrict uc,
                          const real *restrict up, const real *vel,
                          const real *damp, const real *c2, size_t r,
                          size_t nz, size_t nx, size_t ny, real dz, real dx,
                          real dy, real dt)
{
    real dz2 = dz * dz, dx2 = dx * dx, dy2 = dy * dy, dt2 = dt * dt;
    size_t plane = nx * ny;
    #pragma omp parallel for
    for (size_t i = r; i < nz - r; i++) {
        for (size_t j = r; j < nx - r; j++) {
            for (size_t k = r; k < ny - r; k++) {
                size_t p = (i * nx + j) * ny + k;
                real value = 0.0;
                real sy = c2[0] * uc[p], sx = c2[0] * uc[p], sz = c2[0] * uc[p];
                for (size_t q = 1; q <= r; q++) {
                    sy += c2[q] * (uc[p + q] + uc[p - q]);
                    sx += c2[q] * (uc[p + q * ny] + uc[p - q * ny]);
                    sz += c2[q] * (uc[p + q * plane] + uc[p - q * plane]);
                }
                value += sy / dy2 + sx / dx2 + sz / dz2;
                un[p] = leapfrog(value, vel[p], damp[p], dt, dt2, uc[p], up[p]);
            }
        }
    }
}

/* xfd_stride: row stride of the x-axis first derivatives. The reference uses
 * nx (variable_density/3d/wave.c:185-186), the layout needs ny; they agree
 * for nx == ny. */
static void stencil_3d_vd(real *restrict un, const real *restrict uc,
                          const real *restrict up, const real *vel,
                          const real *den, const real *damp, const real *c2,
                          const real *c1, size_t r, size_t nz, size_t nx,
                          size_t ny, real dz, real dx, real dy, real dt,
                          size_t xfd_stride)
{
    real dz2 = dz * dz, dx2 = dx * dx, dy2 = dy * dy, dt2 = dt * dt;
    size_t plane = nx * ny;
    #pragma omp parallel for
    for (size_t i = r; i < nz - r; i++) {
        for (size_t j = r; j < nx - r; j++) {
            for (size_t k = r; k < ny - r; k++) {
                size_t p = (i * nx + j) * ny + k;
                size_t o = p;  /* density index (same grid) */
                real value = 0.0;
                real sdy = c2[0] * uc[p], sdx = c2[0] * uc[p], sdz = c2[0] * uc[p];
                real fuy = 0.0, fux = 0.0, fuz = 0.0;
                real fry = 0.0, frx = 0.0, frz = 0.0;
                for (size_t q = 1; q <= r; q++) {
                    sdy += c2[q] * (uc[p + q] + uc[p - q]);
                    fuy += c1[q] * (uc[p + q] - uc[p - q]);
                    fry += c1[q] * (den[o + q] - den[o - q]);

                    sdx += c2[q] * (uc[p + q * ny] + uc[p - q * ny]);
                    fux += c1[q] * (uc[p + q * xfd_stride] - uc[p - q * xfd_stride]);
                    frx += c1[q] * (den[o + q * xfd_stride] - den[o - q * xfd_stride]);

                    sdz += c2[q] * (uc[p + q * plane] + uc[p - q * plane]);
                    fuz += c1[q] * (uc[p + q * plane] - uc[p - q * plane]);
                    frz += c1[q] * (den[o + q * plane] - den[o - q * plane]);
                }
                value += sdy / dy2 + sdx / dx2 + sdz / dz2;
                real ty = (fuy * fry) / (4 * dy2);
                real tx = (fux * frx) / (4 * dx2);
                real tz = (fuz * frz) / (4 * dz2);
                value -= (ty + tx + tz) / den[o];
                un[p] = leapfrog(value, vel[p], damp[p], dt, dt2, uc[p], up[p]);
            }
        }
    }
}

/* ---- section 2: KWS source injection (wave.c:182-271) ------------------- */

/* Wavelet sample of source `s` at step n (wave.c:199-205). */
static inline real wavelet_sample(const real *w, size_t count, size_t n,
                                  size_t nsrc, size_t s)
{
    return count > 1 ? w[(n - 1) * nsrc + s] : w[n - 1];
}

static void inject_sources(real *un, const real *vel, const real *damp,
                           const real *w, size_t wcount, size_t n,
                           const size_t *iv, const real *val,
                           const size_t *voff, size_t nsrc, int dim,
                           size_t nx, size_t ny, real dt)
{
    real dt2 = dt * dt;
    for (size_t s = 0; s < nsrc; s++) {
        real ws = wavelet_sample(w, wcount, n, nsrc, s);
        if (ws == 0.0)
            continue;
        const size_t *b = iv + s * 2 * (size_t)dim;
        size_t lz = b[1] - b[0] + 1, lx = b[3] - b[2] + 1;
        const real *kz = val + voff[s];
        const real *kx = kz + lz;
        const real *ky = kx + lx;  /* 3D only */
        for (size_t i = b[0]; i <= b[1]; i++) {
            for (size_t j = b[2]; j <= b[3]; j++) {
                if (dim == 2) {
                    real kws = kz[i - b[0]] * kx[j - b[2]];
                    size_t p = i * nx + j;
                    real slowness = 1.0 / (vel[p] * vel[p]);
                    real den = (1.0 + damp[p] * dt / (2 * slowness));
                    un[p] += dt2 / slowness * kws * ws / den;
                } else {
                    for (size_t k = b[4]; k <= b[5]; k++) {
                        real kws = kz[i - b[0]] * kx[j - b[2]] * ky[k - b[4]];
                        size_t p = (i * nx + j) * ny + k;
                        real slowness = 1.0 / (vel[p] * vel[p]);
                        real den = (1.0 + damp[p] * dt / (2 * slowness));
                        un[p] += dt2 / slowness * kws * ws / den;
                    }
                }
            }
        }
    }
}

/* ---- section 3: boundary conditions on u_next (wave.c:274-393) ---------- */

/* One edge of one line: `first` is the index of the first/last interior point
 * on the line, `step` the element stride along the normal, `dir` = -1 for the
 * "before" edge (halo below first) and +1 for "after". */
static inline void edge_bc(real *u, size_t first, size_t step, size_t r,
                           size_t type, int dir)
{
    if (type == BC_DIRICHLET)
        u[first] = 0.0;
    if (type == BC_NEUMANN) {
        for (size_t q = 1; q <= r; q++) {
            if (dir < 0)
                u[first - q * step] = u[first + q * step];
            else
                u[first + q * step] = u[first - q * step];
        }
    }
}

static void boundary_2d(real *u, const size_t *bc, size_t r, size_t nz,
                        size_t nx)
{
    /* x edges over interior rows, then z edges over interior columns */
    #pragma omp parallel for
    for (size_t i = r; i < nz - r; i++) {
        edge_bc(u, i * nx + r, 1, r, bc[2], -1);
        edge_bc(u, i * nx + (nx - r - 1), 1, r, bc[3], +1);
    }
    #pragma omp parallel for
    for (size_t j = r; j < nx - r; j++) {
        edge_bc(u, r * nx + j, nx, r, bc[0], -1);
        edge_bc(u, (nz - r - 1) * nx + j, nx, r, bc[1], +1);
    }
}

static void boundary_3d(real *u, const size_t *bc, size_t r, size_t nz,
                        size_t nx, size_t ny)
{
    size_t plane = nx * ny;
    /* y edges, then x edges, then z edges (3d/wave.c:299-481) */
    #pragma omp parallel for
    for (size_t i = r; i < nz - r; i++)
        for (size_t j = r; j < nx - r; j++) {
            edge_bc(u, (i * nx + j) * ny + r, 1, r, bc[4], -1);
            edge_bc(u, (i * nx + j) * ny + (ny - r - 1), 1, r, bc[5], +1);
        }
    #pragma omp parallel for
    for (size_t i = r; i < nz - r; i++)
        for (size_t k = r; k < ny - r; k++) {
            edge_bc(u, (i * nx + r) * ny + k, ny, r, bc[2], -1);
            edge_bc(u, (i * nx + (nx - r - 1)) * ny + k, ny, r, bc[3], +1);
        }
    #pragma omp parallel for
    for (size_t j = r; j < nx - r; j++)
        for (size_t k = r; k < ny - r; k++) {
            edge_bc(u, (r * nx + j) * ny + k, plane, r, bc[0], -1);
            edge_bc(u, ((nz - r - 1) * nx + j) * ny + k, plane, r, bc[1], +1);
        }
}

/* ---- section 4: receivers (wave.c:395-464) ------------------------------ */

static void record_receivers(real *rec_row, const real *uc, const size_t *iv,
                             const real *val, const size_t *voff, size_t nrec,
                             int dim, size_t nx, size_t ny)
{
    #pragma omp parallel for
    for (size_t s = 0; s < nrec; s++) {
        real sum = 0.0;
        const size_t *b = iv + s * 2 * (size_t)dim;
        size_t lz = b[1] - b[0] + 1, lx = b[3] - b[2] + 1;
        const real *kz = val + voff[s];
        const real *kx = kz + lz;
        const real *ky = kx + lx;
        for (size_t i = b[0]; i <= b[1]; i++)
            for (size_t j = b[2]; j <= b[3]; j++) {
                if (dim == 2) {
                    real kws = kz[i - b[0]] * kx[j - b[2]];
                    sum += uc[i * nx + j] * kws;
                } else {
                    for (size_t k = b[4]; k <= b[5]; k++) {
                        real kws = kz[i - b[0]] * kx[j - b[2]] * ky[k - b[4]];
                        sum += uc[(i * nx + j) * ny + k] * kws;
                    }
                }
            }
        rec_row[s] = sum;
    }
}

/* ---- the time loop ------------------------------------------------------ */

typedef struct {
    int dim, vd;
    size_t xfd_stride;  /* 3D VD only */
    real *u;
    const real *vel, *den, *damp, *w, *c2, *c1;
    size_t wcount;
    const size_t *bc;
    const size_t *siv, *svoff;
    const real *sval;
    const size_t *riv, *rvoff;
    const real *rval;
    real *rec;
    size_t nsrc, nrec, nz, nx, ny;
    real dz, dx, dy, dt;
    size_t stride, begin, end, order;
} problem;

static double run(const problem *P)
{
    double t0 = wall_seconds();
    size_t r = P->order / 2;
    size_t npts = P->nz * P->nx * P->ny;
    slot_state s = {0, 1, 2};
    for (size_t n = P->begin; n <= P->end; n++) {
        slots_at_step(&s, n, P->stride);
        real *un = P->u + s.next * npts;
        const real *uc = P->u + s.cur * npts;
        const real *up = P->u + s.prev * npts;
        if (P->dim == 2 && !P->vd)
            stencil_2d_cd(un, uc, up, P->vel, P->damp, P->c2, r, P->nz, P->nx,
                          P->dz, P->dx, P->dt);
        else if (P->dim == 2)
            stencil_2d_vd(un, uc, up, P->vel, P->den, P->damp, P->c2, P->c1, r,
                          P->nz, P->nx, P->dz, P->dx, P->dt);
        else if (!P->vd)
            stencil_3d_cd(un, uc, up, P->vel, P->damp, P->c2, r, P->nz, P->nx,
                          P->ny, P->dz, P->dx, P->dy, P->dt);
        else
            stencil_3d_vd(un, uc, up, P->vel, P->den, P->damp, P->c2, P->c1, r,
                          P->nz, P->nx, P->ny, P->dz, P->dx, P->dy, P->dt,
                          P->xfd_stride);
        inject_sources(un, P->vel, P->damp, P->w, P->wcount, n, P->siv,
                       P->sval, P->svoff, P->nsrc, P->dim, P->nx, P->ny, P->dt);
        if (P->dim == 2)
            boundary_2d(un, P->bc, r, P->nz, P->nx);
        else
            boundary_3d(un, P->bc, r, P->nz, P->nx, P->ny);
        record_receivers(P->rec + (n - 1) * P->nrec, uc, P->riv, P->rval,
                         P->rvoff, P->nrec, P->dim, P->nx, P->ny);
        if (slots_after_step(&s, n, P->stride, P->end))
            exchange_slots(P->u + s.cur * npts, P->u + s.next * npts, npts);
    }
    return wall_seconds() - t0;
}

/* ---- exported entry points: the reference's `forward` argument order ---- */

double EXPORT(oracle_forward_2d_cd)(
    real *u, real *velocity, real *damp, real *wavelet, size_t wavelet_size,
    size_t wavelet_count, real *coeff, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    real *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, real *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    real *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, real dz, real dx, size_t saving_stride, real dt,
    size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots)
{
    (void)wavelet_size; (void)src_points_interval_size;
    (void)src_points_values_size; (void)rec_points_interval_size;
    (void)rec_points_values_size; (void)num_snapshots;
    problem P = {2, 0, 0, u, velocity, NULL, damp, wavelet, coeff, NULL,
                 wavelet_count, boundary_conditions, src_points_interval,
                 src_points_values_offset, src_points_values,
                 rec_points_interval, rec_points_values_offset,
                 rec_points_values, receivers, num_sources, num_receivers, nz,
                 nx, 1, dz, dx, 1, dt, saving_stride, begin_timestep,
                 end_timestep, space_order};
    return run(&P);
}

double EXPORT(oracle_forward_2d_vd)(
    real *u, real *velocity, real *density, real *damp, real *wavelet,
    size_t wavelet_size, size_t wavelet_count, real *coeff_order2,
    real *coeff_order1, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    real *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, real *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    real *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, real dz, real dx, size_t saving_stride, real dt,
    size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots)
{
    (void)wavelet_size; (void)src_points_interval_size;
    (void)src_points_values_size; (void)rec_points_interval_size;
    (void)rec_points_values_size; (void)num_snapshots;
    problem P = {2, 1, 0, u, velocity, density, damp, wavelet, coeff_order2,
                 coeff_order1, wavelet_count, boundary_conditions,
                 src_points_interval, src_points_values_offset,
                 src_points_values, rec_points_interval,
                 rec_points_values_offset, rec_points_values, receivers,
                 num_sources, num_receivers, nz, nx, 1, dz, dx, 1, dt,
                 saving_stride, begin_timestep, end_timestep, space_order};
    return run(&P);
}

double EXPORT(oracle_forward_3d_cd)(
    real *u, real *velocity, real *damp, real *wavelet, size_t wavelet_size,
    size_t wavelet_count, real *coeff, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    real *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, real *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    real *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, size_t ny, real dz, real dx, real dy, size_t saving_stride,
    real dt, size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots)
{
    (void)wavelet_size; (void)src_points_interval_size;
    (void)src_points_values_size; (void)rec_points_interval_size;
    (void)rec_points_values_size; (void)num_snapshots;
    problem P = {3, 0, 0, u, velocity, NULL, damp, wavelet, coeff, NULL,
                 wavelet_count, boundary_conditions, src_points_interval,
                 src_points_values_offset, src_points_values,
                 rec_points_interval, rec_points_values_offset,
                 rec_points_values, receivers, num_sources, num_receivers, nz,
                 nx, ny, dz, dx, dy, dt, saving_stride, begin_timestep,
                 end_timestep, space_order};
    return run(&P);
}

static double forward_3d_vd(
    size_t xfd_stride_is_ny, real *u, real *velocity, real *density,
    real *damp, real *wavelet, size_t wavelet_count, real *coeff_order2,
    real *coeff_order1, size_t *boundary_conditions,
    size_t *src_points_interval, real *src_points_values,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    real *rec_points_values, size_t *rec_points_values_offset,
    real *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, size_t ny, real dz, real dx, real dy, size_t saving_stride,
    real dt, size_t begin_timestep, size_t end_timestep, size_t space_order)
{
    problem P = {3, 1, xfd_stride_is_ny ? ny : nx, u, velocity, density, damp,
                 wavelet, coeff_order2, coeff_order1, wavelet_count,
                 boundary_conditions, src_points_interval,
                 src_points_values_offset, src_points_values,
                 rec_points_interval, rec_points_values_offset,
                 rec_points_values, receivers, num_sources, num_receivers, nz,
                 nx, ny, dz, dx, dy, dt, saving_stride, begin_timestep,
                 end_timestep, space_order};
    return run(&P);
}

/* The reference's 3D variable-density operator, x first derivatives with
 * row stride nx (variable_density/3d/wave.c:185-186). */
double EXPORT(oracle_forward_3d_vd)(
    real *u, real *velocity, real *density, real *damp, real *wavelet,
    size_t wavelet_size, size_t wavelet_count, real *coeff_order2,
    real *coeff_order1, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    real *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, real *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    real *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, size_t ny, real dz, real dx, real dy, size_t saving_stride,
    real dt, size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots)
{
    (void)wavelet_size; (void)src_points_interval_size;
    (void)src_points_values_size; (void)rec_points_interval_size;
    (void)rec_points_values_size; (void)num_snapshots;
    return forward_3d_vd(0, u, velocity, density, damp, wavelet, wavelet_count,
                         coeff_order2, coeff_order1, boundary_conditions,
                         src_points_interval, src_points_values,
                         src_points_values_offset, rec_points_interval,
                         rec_points_values, rec_points_values_offset,
                         receivers, num_sources, num_receivers, nz, nx, ny, dz,
                         dx, dy, saving_stride, dt, begin_timestep,
                         end_timestep, space_order);
}

/* Same operator with the x first derivatives on the layout's row stride ny,
 * the operator the GPU library implements; identical to the above when
 * nx == ny. */
double EXPORT(oracle_forward_3d_vdfix)(
    real *u, real *velocity, real *density, real *damp, real *wavelet,
    size_t wavelet_size, size_t wavelet_count, real *coeff_order2,
    real *coeff_order1, size_t *boundary_conditions,
    size_t *src_points_interval, size_t src_points_interval_size,
    real *src_points_values, size_t src_points_values_size,
    size_t *src_points_values_offset, size_t *rec_points_interval,
    size_t rec_points_interval_size, real *rec_points_values,
    size_t rec_points_values_size, size_t *rec_points_values_offset,
    real *receivers, size_t num_sources, size_t num_receivers, size_t nz,
    size_t nx, size_t ny, real dz, real dx, real dy, size_t saving_stride,
    real dt, size_t begin_timestep, size_t end_timestep, size_t space_order,
    size_t num_snapshots)
{
    (void)wavelet_size; (void)src_points_interval_size;
    (void)src_points_values_size; (void)rec_points_interval_size;
    (void)rec_points_values_size; (void)num_snapshots;
    return forward_3d_vd(1, u, velocity, density, damp, wavelet, wavelet_count,
                         coeff_order2, coeff_order1, boundary_conditions,
                         src_points_interval, src_points_values,
                         src_points_values_offset, rec_points_interval,
                         rec_points_values, rec_points_values_offset,
                         receivers, num_sources, num_receivers, nz, nx, ny, dz,
                         dx, dy, saving_stride, dt, begin_timestep,
                         end_timestep, space_order);
}
