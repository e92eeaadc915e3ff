/*
 * sw_forward_shim.c -- `forward` symbol for one (dimension, density,
 * precision) variant, so that the reference's Middleware can load this
 * library exactly as it loads a compiled wave.c (middleware.py:26-51,
 * 142-154: `lib.forward` with argtypes built from the call's values).
 *
 * Built once per variant with -DSW_DIM=2|3 -DSW_VD=0|1 -DSW_F64=0|1 into
 * libsimwave_forward_<d>d_<cd|vd>_<f32|f64>.so, linked to libsimwave_gb300.so.
 */
#include <stddef.h>

#include "simwave_gb300.h"

#if SW_F64
typedef double real;
#define PREC f64
#else
typedef float real;
#define PREC f32
#endif

#define JOIN3_(a, b, c) simwave_forward_##a##_##b##_##c
#define JOIN3(a, b, c) JOIN3_(a, b, c)

#if SW_DIM == 2
#define DIMTAG 2d
#define GRID_ARGS size_t nz, size_t nx, real dz, real dx
#define GRID_PASS nz, nx, dz, dx
#else
#define DIMTAG 3d
#define GRID_ARGS size_t nz, size_t nx, size_t ny, real dz, real dx, real dy
#define GRID_PASS nz, nx, ny, dz, dx, dy
#endif

#if SW_VD
#define DENTAG vd
#define MODEL_ARGS real *velocity, real *density, real *damp
#define MODEL_PASS velocity, density, damp
#define COEFF_ARGS real *coeff_order2, real *coeff_order1
#define COEFF_PASS coeff_order2, coeff_order1
#else
#define DENTAG cd
#define MODEL_ARGS real *velocity, real *damp
#define MODEL_PASS velocity, damp
#define COEFF_ARGS real *coeff
#define COEFF_PASS coeff
#endif

double forward(real *u, MODEL_ARGS, real *wavelet, size_t wavelet_size,
               size_t wavelet_count, COEFF_ARGS, size_t *boundary_conditions,
               size_t *src_points_interval, size_t src_points_interval_size,
               real *src_points_values, size_t src_points_values_size,
               size_t *src_points_values_offset, size_t *rec_points_interval,
               size_t rec_points_interval_size, real *rec_points_values,
               size_t rec_points_values_size,
               size_t *rec_points_values_offset, real *receivers,
               size_t num_sources, size_t num_receivers, GRID_ARGS,
               size_t saving_stride, real dt, size_t begin_timestep,
               size_t end_timestep, size_t space_order, size_t num_snapshots)
{
    return JOIN3(DIMTAG, DENTAG, PREC)(
        u, MODEL_PASS, wavelet, wavelet_size, wavelet_count, COEFF_PASS,
        boundary_conditions, src_points_interval, src_points_interval_size,
        src_points_values, src_points_values_size, src_points_values_offset,
        rec_points_interval, rec_points_interval_size, rec_points_values,
        rec_points_values_size, rec_points_values_offset, receivers,
        num_sources, num_receivers, GRID_PASS, saving_stride, dt,
        begin_timestep, end_timestep, space_order, num_snapshots);
}
