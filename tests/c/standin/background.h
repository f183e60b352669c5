/* Stand-in for the reference's src/background.h (coffe_background_t,
   background.h:23-45): the splines, with the reference's field names. */
#ifndef COFFE_BACKGROUND_H
#define COFFE_BACKGROUND_H

#include "common.h"

typedef struct coffe_background_t {
    coffe_interpolation z_as_chi;
    coffe_interpolation a;
    coffe_interpolation Hz;
    coffe_interpolation conformal_Hz;
    coffe_interpolation conformal_Hz_prime;
    coffe_interpolation D1;
    coffe_interpolation f;
    coffe_interpolation G1, G2;
    coffe_interpolation comoving_distance;
    int flag;
} coffe_background_t;

#endif
