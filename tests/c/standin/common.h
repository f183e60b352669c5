/*
 * Stand-in for the reference's src/common.h, for compiling
 * coffe_gb300/shim/coffe_gpu_shim.c in this repository's tests without the
 * reference (or GSL).  The types carry the reference's type and field names
 * (coffe_interpolation, common.h:228-232; coffe_parameters_t, common.h:340-550;
 * coffe_multipoles_coords_t, common.h:178-183) and gsl_spline its public fields
 * (x, y, size), so that the shim compiles unchanged against either; only the
 * fields the shim reads are declared.
 */
#ifndef COFFE_COMMON_H
#define COFFE_COMMON_H

#include <stddef.h>

typedef struct {
    void *interp;
    double *x;
    double *y;
    size_t size;
} gsl_spline;

typedef struct {
    size_t cache;
} gsl_interp_accel;

typedef struct coffe_interpolation {
    gsl_spline *spline;
    gsl_interp_accel *accel;
} coffe_interpolation;

typedef struct coffe_interpolation2d {
    void *spline;
    void *xaccel, *yaccel;
} coffe_interpolation2d;

enum coffe_interp1d_type {
    COFFE_INTERP_LINEAR = 1,
    COFFE_INTERP_POLYNOMIAL = 2,
    COFFE_INTERP_CSPLINE = 3,
    COFFE_INTERP_CSPLINE_PERIODIC = 4,
    COFFE_INTERP_AKIMA = 5,
    COFFE_INTERP_AKIMA_PERIODIC = 6,
    COFFE_INTERP_STEFFEN = 7
};

typedef struct coffe_correlation_contributions {
    int den, rsd, len, d1, d2, g1, g2, g3, g4, g5;
} coffe_correlation_contributions;

typedef struct coffe_multipoles_coords_t {
    double z_mean;
    double separation;
    int l;
} coffe_multipoles_coords_t;

typedef struct coffe_parameters_t {
    coffe_correlation_contributions correlation_contrib;
    int bessel_bins;
    double Omega0_cdm;
    double Omega0_baryon;
    double *z_mean;
    size_t z_mean_len;
    double *sep;
    size_t sep_len;
    coffe_interpolation power_spectrum_norm;
    double k_min_norm;
    double k_max_norm;
    enum coffe_interp1d_type interp_method;
    int *multipole_values;
    size_t multipole_values_len;
    int flatsky_local;
    int flatsky_local_nonlocal;
    int flatsky_nonlocal;
    double h;
    int only_cross_correlations;
    double integration_1d_prec;
} coffe_parameters_t;

void *coffe_malloc(size_t size);

int coffe_init_spline(coffe_interpolation *interp, const double *xi, const double *yi,
                      const size_t bins, const enum coffe_interp1d_type interpolation_type);

#endif
