/*
 * Runs the sequence a reference C caller runs (src/main.c:138-151), with the
 * drivers of coffe_gb300/shim/coffe_gpu_shim.c in place of the CPU ones:
 * a background the caller built (its splines' nodes), the power spectrum,
 * coffe_integrals_init_gpu, then coffe_multipoles_init_gpu, and writes the
 * integral tables and the multipole array out for comparison with the oracle.
 *
 * usage: shim_test <input> <output>
 * input (native-endian): 8 int64 header values
 *   nk, n_bg, n_z, n_l, n_sep, bessel_bins, contrib mask (1 den, 2 rsd, 4 len),
 *   precision (0 FP64, 1 mixed)
 * then doubles: k[nk], pk[nk], z[n_bg], chi[n_bg], D1[n_bg], f[n_bg], a[n_bg],
 *   conformal_H[n_bg], z_mean[n_z], l[n_l] (as doubles), sep[n_sep],
 *   Omega0_cdm, Omega0_baryon, h, integration_1d_prec.
 * output: int64 number of tables, then per table int64 (n, l, length) and the
 *   x and y arrays; int64 number of multipoles, then (z_mean, l, sep, value) as
 *   doubles per multipole, in the array's order.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "coffe_gpu_shim.h"

static double *read_doubles(FILE *f, size_t n)
{
    double *p = (double *)coffe_malloc(sizeof(double) * (n ? n : 1));
    if (fread(p, sizeof(double), n, f) != n) {
        fprintf(stderr, "shim_test: short input\n");
        exit(2);
    }
    return p;
}

static void put_i64(FILE *f, int64_t v) { fwrite(&v, sizeof v, 1, f); }

int main(int argc, char **argv)
{
    int64_t hdr[8];
    FILE *in, *out;
    size_t i, nk, nbg, nz, nl, ns;
    double *k, *pk, *z, *chi, *D1, *fg, *a, *cH, *lv, *tail;
    coffe_parameters_t par = {0};
    coffe_background_t bg = {0};
    coffe_integral_array_t integral = {0};
    coffe_multipoles_array_t mp = {0};

    if (argc != 3) {
        fprintf(stderr, "usage: shim_test <input> <output>\n");
        return 2;
    }
    in = fopen(argv[1], "rb");
    if (!in || fread(hdr, sizeof(int64_t), 8, in) != 8) {
        fprintf(stderr, "shim_test: cannot read %s\n", argv[1]);
        return 2;
    }
    nk = (size_t)hdr[0];
    nbg = (size_t)hdr[1];
    nz = (size_t)hdr[2];
    nl = (size_t)hdr[3];
    ns = (size_t)hdr[4];
    k = read_doubles(in, nk);
    pk = read_doubles(in, nk);
    z = read_doubles(in, nbg);
    chi = read_doubles(in, nbg);
    D1 = read_doubles(in, nbg);
    fg = read_doubles(in, nbg);
    a = read_doubles(in, nbg);
    cH = read_doubles(in, nbg);
    par.z_mean = read_doubles(in, nz);
    lv = read_doubles(in, nl);
    par.sep = read_doubles(in, ns);
    tail = read_doubles(in, 4);
    fclose(in);

    par.z_mean_len = nz;
    par.sep_len = ns;
    par.multipole_values = (int *)coffe_malloc(sizeof(int) * (nl ? nl : 1));
    for (i = 0; i < nl; ++i) par.multipole_values[i] = (int)lv[i];
    par.multipole_values_len = nl;
    par.bessel_bins = (int)hdr[5];
    par.correlation_contrib.den = (hdr[6] & 1) != 0;
    par.correlation_contrib.rsd = (hdr[6] & 2) != 0;
    par.correlation_contrib.len = (hdr[6] & 4) != 0;
    par.Omega0_cdm = tail[0];
    par.Omega0_baryon = tail[1];
    par.h = tail[2];
    par.integration_1d_prec = tail[3];
    par.interp_method = COFFE_INTERP_AKIMA;
    coffe_init_spline(&par.power_spectrum_norm, k, pk, nk, COFFE_INTERP_CSPLINE);
    par.k_min_norm = k[0];
    par.k_max_norm = k[nk - 1];
    /* the caller's background: every spline on the same z nodes */
    coffe_init_spline(&bg.comoving_distance, z, chi, nbg, par.interp_method);
    coffe_init_spline(&bg.D1, z, D1, nbg, par.interp_method);
    coffe_init_spline(&bg.f, z, fg, nbg, par.interp_method);
    coffe_init_spline(&bg.a, z, a, nbg, par.interp_method);
    coffe_init_spline(&bg.conformal_Hz, z, cH, nbg, par.interp_method);
    coffe_init_spline(&bg.z_as_chi, chi, z, nbg, par.interp_method);
    coffe_gpu_shim_set_precision((int)hdr[7]);

    if (coffe_integrals_init_gpu(&par, &bg, &integral) != EXIT_SUCCESS) return 1;
    if (coffe_multipoles_init_gpu(&par, &bg, &integral, &mp) != EXIT_SUCCESS) return 1;

    out = fopen(argv[2], "wb");
    if (!out) return 2;
    put_i64(out, (int64_t)integral.size);
    for (i = 0; i < integral.size; ++i) {
        const gsl_spline *s = integral.array[i].result.spline;
        put_i64(out, integral.array[i].n);
        put_i64(out, integral.array[i].l);
        put_i64(out, (int64_t)s->size);
        fwrite(s->x, sizeof(double), s->size, out);
        fwrite(s->y, sizeof(double), s->size, out);
    }
    put_i64(out, (int64_t)mp.size);
    for (i = 0; i < mp.size; ++i) {
        const double rec[4] = {mp.array[i].coords.z_mean, (double)mp.array[i].coords.l,
                               mp.array[i].coords.separation, mp.array[i].value};
        fwrite(rec, sizeof(double), 4, out);
    }
    fclose(out);
    coffe_integrals_free(&integral);
    coffe_multipoles_free(&mp);
    coffe_gpu_shim_release();
    free(k);
    free(pk);
    free(z);
    free(chi);
    free(D1);
    free(fg);
    free(a);
    free(cH);
    free(lv);
    free(tail);
    return 0;
}
