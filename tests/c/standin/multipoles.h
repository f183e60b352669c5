/* Stand-in for the reference's src/multipoles.h (coffe_multipoles_t and
   coffe_multipoles_array_t, multipoles.h:27-41). */
#ifndef COFFE_MULTIPOLES_H
#define COFFE_MULTIPOLES_H

#include "common.h"

typedef struct coffe_multipoles_t {
    coffe_multipoles_coords_t coords;
    double value;
} coffe_multipoles_t;

typedef struct coffe_multipoles_array_t {
    coffe_multipoles_t *array;
    size_t size;
} coffe_multipoles_array_t;

int coffe_multipoles_free(coffe_multipoles_array_t *mp);

#endif
