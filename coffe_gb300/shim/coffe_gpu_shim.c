/*
 * coffe_gpu_shim.c -- the reference's integral and multipole drivers on the GPU
 * (declarations and build notes in coffe_gpu_shim.h).  Plain C99: it reads the
 * reference's own structures (coffe_parameters_t, common.h:340-550;
 * coffe_background_t, background.h:23-45; coffe_integral_array_t,
 * integrals.h:25-52; coffe_multipoles_array_t, multipoles.h:27-41) and writes the
 * same outputs the CPU drivers write.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "coffe_gpu.h"
#include "coffe_gpu_shim.h"

static coffe_gpu_ctx_t *shim_ctx = NULL; /* one context per process, device 0 */
static int shim_precision = COFFE_GPU_FP64;

/* the default full-sky terms of coffe_integrals_init (integrals.c:599-608);
   the first three are all the density and RSD terms read */
static const int shim_n[8] = {0, 0, 0, 1, 1, 2, 2, 3};
static const int shim_l[8] = {0, 2, 4, 1, 3, 0, 2, 1};

static int shim_fail(const char *what, int status)
{
    fprintf(stderr, "coffe_gpu: %s: %s (%s)\n", what, coffe_gpu_strerror(status),
            shim_ctx ? coffe_gpu_last_error(shim_ctx) : "no context");
    return EXIT_FAILURE;
}

static int shim_context(void)
{
    int st;
    if (shim_ctx) return EXIT_SUCCESS;
    st = coffe_gpu_ctx_create(0, &shim_ctx);
    if (st != COFFE_GPU_OK) {
        shim_ctx = NULL;
        return shim_fail("coffe_gpu_ctx_create", st);
    }
    return EXIT_SUCCESS;
}

void coffe_gpu_shim_set_precision(int precision)
{
    shim_precision = precision == COFFE_GPU_MIXED ? COFFE_GPU_MIXED : COFFE_GPU_FP64;
}

void coffe_gpu_shim_release(void)
{
    if (shim_ctx) coffe_gpu_ctx_destroy(shim_ctx);
    shim_ctx = NULL;
}

static int shim_uses_lensing(const coffe_parameters_t *par)
{
    return par->correlation_contrib.len != 0;
}

int coffe_integrals_init_gpu(const coffe_parameters_t *par, const coffe_background_t *bg,
                             coffe_integral_array_t *integral)
{
    const gsl_spline *pk = par->power_spectrum_norm.spline;
    const int n_terms = shim_uses_lensing(par) ? 8 : 3;
    const size_t N = (size_t)par->bessel_bins;
    size_t len, t;
    double *x, *y;
    int st;
    (void)bg; /* the tables do not depend on the background */
    if (!pk || pk->size < 2) {
        fprintf(stderr, "coffe_gpu: no power spectrum\n");
        return EXIT_FAILURE;
    }
    if (N < 64 || N > 16384 || (N & (N - 1)) != 0) {
        fprintf(stderr, "coffe_gpu: bessel_bins = %d is not a power of two in [64, 16384]\n",
                par->bessel_bins);
        return EXIT_FAILURE;
    }
    /* the FFTLog grid spans [k_min_norm, k_max_norm] (integrals.c:648-649); the
       GPU takes it from the spectrum's first and last k */
    if (par->k_min_norm < pk->x[0] * (1 - 1e-12) || par->k_min_norm > pk->x[0] * (1 + 1e-12) ||
        par->k_max_norm < pk->x[pk->size - 1] * (1 - 1e-12) ||
        par->k_max_norm > pk->x[pk->size - 1] * (1 + 1e-12)) {
        fprintf(stderr, "coffe_gpu: k_min_norm, k_max_norm must be the spectrum's first and "
                        "last k\n");
        return EXIT_FAILURE;
    }
    if (shim_context() != EXIT_SUCCESS) return EXIT_FAILURE;
    st = coffe_gpu_integrals_init(shim_ctx, pk->x, pk->y, 1, pk->size, shim_n, shim_l, n_terms,
                                  N, shim_precision, COFFE_GPU_SMALL_R);
    if (st != COFFE_GPU_OK) return shim_fail("coffe_gpu_integrals_init", st);

    /* the same (x, y) arrays the CPU driver splines (integrals.c:652-658), so
       every later coffe_interp_spline(&integral->array[i].result, r) is unchanged */
    coffe_integrals_free(integral);
    integral->array = (coffe_integral_t *)coffe_malloc(sizeof(coffe_integral_t) * n_terms);
    integral->size = (size_t)n_terms;
    len = coffe_gpu_integral_table_len(N);
    x = (double *)malloc(sizeof(double) * len);
    y = (double *)malloc(sizeof(double) * len);
    if (!x || !y) {
        free(x);
        free(y);
        fprintf(stderr, "coffe_gpu: out of host memory\n");
        return EXIT_FAILURE;
    }
    for (t = 0; t < (size_t)n_terms; ++t) {
        coffe_integral_new(&integral->array[t]);
        integral->array[t].n = shim_n[t];
        integral->array[t].l = shim_l[t];
        integral->array[t].state_n = COFFE_INTEGER;
        integral->array[t].state_l = COFFE_INTEGER;
        st = coffe_gpu_integral_get(shim_ctx, 0, (int)t, x, y);
        if (st != COFFE_GPU_OK) {
            free(x);
            free(y);
            return shim_fail("coffe_gpu_integral_get", st);
        }
        coffe_init_spline(&integral->array[t].result, x, y, len, par->interp_method);
    }
    free(x);
    free(y);
    return EXIT_SUCCESS;
}

int coffe_multipoles_init_gpu(coffe_parameters_t *par, coffe_background_t *bg,
                              coffe_integral_array_t *integral, coffe_multipoles_array_t *mp)
{
    const size_t nz = par->z_mean_len, nl = par->multipole_values_len, ns = par->sep_len;
    const gsl_spline *chi = bg->comoving_distance.spline;
    int contrib = 0, st = COFFE_GPU_OK;
    int *spec = NULL;
    int64_t *off = NULL;
    double *sep = NULL, *out = NULL;
    size_t i, j, k, c;
    (void)integral; /* the tables of coffe_integrals_init_gpu live on the device */
    if (par->correlation_contrib.d1 || par->correlation_contrib.d2 || par->correlation_contrib.g1 ||
        par->correlation_contrib.g2 || par->correlation_contrib.g3 ||
        par->correlation_contrib.g4 || par->correlation_contrib.g5 || par->flatsky_local) {
        fprintf(stderr, "coffe_gpu: only the den, rsd and len contributions run on the GPU\n");
        return EXIT_FAILURE;
    }
    if (par->correlation_contrib.den) contrib |= COFFE_GPU_DEN;
    if (par->correlation_contrib.rsd) contrib |= COFFE_GPU_RSD;
    if (par->correlation_contrib.len) contrib |= COFFE_GPU_LEN;
    if (par->only_cross_correlations) contrib |= COFFE_GPU_ONLY_CROSS;
    if (!(contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD | COFFE_GPU_LEN)) || !chi) {
        fprintf(stderr, "coffe_gpu: nothing to compute\n");
        return EXIT_FAILURE;
    }
    if (shim_context() != EXIT_SUCCESS) return EXIT_FAILURE;

    /* the background the reference built (background.c:301-696): every spline
       is tabulated on the same z nodes (background.c:545-617) */
    st = coffe_gpu_background_set(shim_ctx, chi->x, chi->y, bg->D1.spline->y, bg->f.spline->y,
                                  bg->a.spline->y, bg->conformal_Hz.spline->y, chi->size,
                                  par->Omega0_cdm + par->Omega0_baryon, par->h);
    if (st != COFFE_GPU_OK) return shim_fail("coffe_gpu_background_set", st);
    st = coffe_gpu_set_flatsky(shim_ctx, par->flatsky_local_nonlocal, par->flatsky_nonlocal);
    if (st != COFFE_GPU_OK) return shim_fail("coffe_gpu_set_flatsky", st);

    /* one request per z_mean, each with the full separation list */
    spec = (int *)calloc(nz + 1, sizeof(int));
    off = (int64_t *)malloc(sizeof(int64_t) * (nz + 1));
    sep = (double *)malloc(sizeof(double) * (nz * ns + 1));
    out = (double *)malloc(sizeof(double) * (nz * ns * nl + 1));
    if (!spec || !off || !sep || !out) {
        fprintf(stderr, "coffe_gpu: out of host memory\n");
        st = COFFE_GPU_ENOMEM;
        goto done;
    }
    for (i = 0; i <= nz; ++i) off[i] = (int64_t)(i * ns);
    for (i = 0; i < nz; ++i) memcpy(sep + i * ns, par->sep, sizeof(double) * ns);
    st = coffe_gpu_multipoles(shim_ctx, contrib, shim_precision, par->integration_1d_prec,
                              (int)nz, spec, par->z_mean, off, sep, (int)nl,
                              par->multipole_values, out, 0);
    if (st != COFFE_GPU_OK) {
        shim_fail("coffe_gpu_multipoles", st);
        goto done;
    }

    /* the reference's output order (z_mean, l, sep), multipoles.c:76-86; the
       GPU writes one row of n_l values per separation */
    coffe_multipoles_free(mp);
    mp->size = nz * nl * ns;
    mp->array = (coffe_multipoles_t *)coffe_malloc(sizeof(coffe_multipoles_t) * (mp->size + 1));
    c = 0;
    for (i = 0; i < nz; ++i)
        for (j = 0; j < nl; ++j)
            for (k = 0; k < ns; ++k, ++c) {
                mp->array[c].coords.z_mean = par->z_mean[i];
                mp->array[c].coords.l = par->multipole_values[j];
                mp->array[c].coords.separation = par->sep[k];
                mp->array[c].value = out[(i * ns + k) * nl + j];
            }
done:
    free(spec);
    free(off);
    free(sep);
    free(out);
    return st == COFFE_GPU_OK ? EXIT_SUCCESS : EXIT_FAILURE;
}
