/* Dense real matrix of the reference's math layer (layout of the reference's
 * include/matrix.h:24-31): rows x cols doubles, row-major data[r * cols + c],
 * owned by the caller and released with the reference's matrix_free
 * (free(data), then zero the struct).  The incidence products of
 * incidence.h fill one; the library allocates data with calloc. */
#ifndef PEEC_MATRIX_H
#define PEEC_MATRIX_H

#include <stddef.h>

typedef struct {
    size_t rows;
    size_t cols;
    double *data;
} Matrix;

#endif
