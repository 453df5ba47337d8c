/*
 * Interleaved double-precision complex scalar, layout-compatible with the
 * reference's `Complex` (include/complex_matrix.h:21-26 of the reference
 * project): {re, im}, 16 bytes, no padding.  Only the type lives here.
 */
#ifndef PEEC_COMPLEX_MATRIX_H
#define PEEC_COMPLEX_MATRIX_H

#include <stddef.h>

typedef struct
{
    double re;
    double im;
} Complex;

#endif
