/* Stand-in for the reference's src/integrals.h (coffe_integral_t and
   coffe_integral_array_t, integrals.h:25-52). */
#ifndef COFFE_INTEGRALS_H
#define COFFE_INTEGRALS_H

#include "common.h"

enum coffe_integer_state { COFFE_INTEGER, COFFE_HALF_INTEGER };

typedef struct coffe_integral_t {
    coffe_interpolation result;
    coffe_interpolation2d result2d;
    coffe_interpolation2d renormalization;
    coffe_interpolation renormalization_zero_separation;
    int n, l;
    enum coffe_integer_state state_n, state_l;
} coffe_integral_t;

typedef struct coffe_integral_array_t {
    coffe_integral_t *array;
    size_t size;
} coffe_integral_array_t;

int coffe_integral_new(coffe_integral_t *integral);
int coffe_integrals_free(coffe_integral_array_t *integral);

#endif
