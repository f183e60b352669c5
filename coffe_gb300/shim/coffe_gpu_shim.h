/*
 * coffe_gpu_shim.h -- drop-in replacements for COFFE's coffe_integrals_init
 * (src/integrals.c:580) and coffe_multipoles_init (src/multipoles.c:48) that run
 * on the GPU through include/coffe_gpu.h.
 *
 * A maintainer of the reference compiles coffe_gpu_shim.c beside its src/ files (it
 * includes the reference's own common.h, background.h, integrals.h and
 * multipoles.h), links -lcoffe_gpu, and calls the *_gpu drivers where
 * src/main.c:145-151 and python/coffe/coffe.pyx:3548-3563 call the CPU ones.
 * Same arguments, same outputs (the coffe_integral_t splines, the
 * coffe_multipoles_t array in the reference's (z_mean, l, sep) order,
 * multipoles.c:76-86).  Errors print a message on stderr and return
 * EXIT_FAILURE; the reference's drivers exit() instead.
 */
#ifndef COFFE_GPU_SHIM_H
#define COFFE_GPU_SHIM_H

#include "common.h"
#include "background.h"
#include "integrals.h"
#include "multipoles.h"

#ifdef __cplusplus
extern "C" {
#endif

/* coffe_integrals_init (integrals.c:580-770) for the full-sky integer terms:
   I^0_0, I^0_2, I^0_4, plus I^1_1, I^1_3, I^2_0, I^2_2, I^3_1 when the lensing
   contribution is on.  par->bessel_bins must be a power of two in [64, 16384],
   and par->k_min_norm, par->k_max_norm the first and last k of
   par->power_spectrum_norm (as Coffe.set_power_spectrum_linear sets them). */
int coffe_integrals_init_gpu(const coffe_parameters_t *par, const coffe_background_t *bg,
                             coffe_integral_array_t *integral);

/* coffe_multipoles_init (multipoles.c:48-136): every (z_mean, l, sep) of par in
   one batched launch; den, rsd (and len) contributions. */
int coffe_multipoles_init_gpu(coffe_parameters_t *par, coffe_background_t *bg,
                              coffe_integral_array_t *integral, coffe_multipoles_array_t *mp);

/* COFFE_GPU_FP64 (default) or COFFE_GPU_MIXED for the calls that follow. */
void coffe_gpu_shim_set_precision(int precision);

/* Releases the shim's GPU context (one per process, created on first use). */
void coffe_gpu_shim_release(void);

#ifdef __cplusplus
}
#endif
#endif /* COFFE_GPU_SHIM_H */
