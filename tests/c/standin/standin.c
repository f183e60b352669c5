/* Minimal bodies for the stand-in headers: a "spline" keeps copies of its
   nodes, which is all the shim test reads back. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "background.h"
#include "common.h"
#include "integrals.h"
#include "multipoles.h"

void *coffe_malloc(size_t size)
{
    void *p = malloc(size ? size : 1);
    if (!p) {
        fprintf(stderr, "out of memory\n");
        exit(EXIT_FAILURE);
    }
    return p;
}

int coffe_init_spline(coffe_interpolation *interp, const double *xi, const double *yi,
                      const size_t bins, const enum coffe_interp1d_type interpolation_type)
{
    gsl_spline *s = (gsl_spline *)coffe_malloc(sizeof(gsl_spline));
    (void)interpolation_type;
    s->interp = NULL;
    s->size = bins;
    s->x = (double *)coffe_malloc(sizeof(double) * bins);
    s->y = (double *)coffe_malloc(sizeof(double) * bins);
    memcpy(s->x, xi, sizeof(double) * bins);
    memcpy(s->y, yi, sizeof(double) * bins);
    interp->spline = s;
    interp->accel = NULL;
    return EXIT_SUCCESS;
}

static void spline_free(coffe_interpolation *interp)
{
    if (interp->spline) {
        free(interp->spline->x);
        free(interp->spline->y);
        free(interp->spline);
    }
    interp->spline = NULL;
}

int coffe_integral_new(coffe_integral_t *integral)
{
    memset(integral, 0, sizeof(*integral));
    return EXIT_SUCCESS;
}

int coffe_integrals_free(coffe_integral_array_t *integral)
{
    size_t i;
    for (i = 0; i < integral->size; ++i) spline_free(&integral->array[i].result);
    free(integral->array);
    integral->array = NULL;
    integral->size = 0;
    return EXIT_SUCCESS;
}

int coffe_multipoles_free(coffe_multipoles_array_t *mp)
{
    free(mp->array);
    mp->array = NULL;
    mp->size = 0;
    return EXIT_SUCCESS;
}
