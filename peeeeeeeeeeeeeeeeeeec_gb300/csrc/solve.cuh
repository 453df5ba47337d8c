// Internal entry points of the wavefront triangular solve (lu.cu) for the
// other translation units of the library.
#pragma once

#include <stddef.h>

namespace peec {

// Flag words the solve of n unknowns with nrhs right-hand sides needs.
size_t wave_flag_words_real(int n, int nrhs);
// Doubles of the diagonal-block inverses of an n x n factor.
size_t wave_dinv_words_real(int n);
// Computes the diagonal-block inverses of a packed real LU factor.
bool wave_prepare_real(const double *lu, int n, double *dinv);

// x = U^-1 L^-1 (b permuted by perm) for a packed real LU factor and its
// diagonal-block inverses, enqueued on the calling thread's stream (flags:
// wave_flag_words_real words, err: one int, zero on entry; a timed-out wait
// leaves 6 in *err).  x != b.
bool wave_solve_real(const double *lu, const double *dinv, const int *perm, int n, const double *b, double *x,
                     int nrhs, unsigned *flags, int *err);

}  // namespace peec
