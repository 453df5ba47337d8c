// The graph form of the mixed-precision solve, shared by the LU (lu.cu) and
// the batched frequency sweep (sweep.cu).
#pragma once

#include <stddef.h>

#include "../../include/complex_matrix.h"

namespace peec {

// A mixed solve recorded into a CUDA graph: no host reads, syncs or
// host-side decisions inside.  The FP32 factorisation uses split_terms (3 or
// 6) split-BF16 products and the pivot limit 1e-14 (the power-of-two
// equilibration leaves the largest entry in [1, 2 sqrt 2)), then up to
// `sweeps` FP64 refinement sweeps run from x = 0: all are recorded, and once
// a sweep's componentwise backward error is <= tol a device flag turns the
// later ones into no-ops.  The last backward error (IEEE bits) goes to
// *d_eta_bits and the status (0, or the factorisation's / triangular
// solve's error code) to *d_status, for the host to read after the graph
// has run.  (With 32 or more right-hand sides every sweep runs.)
struct MixedCapture {
    int split_terms;
    int sweeps;
    double tol;
    unsigned long long *d_eta_bits;
    int *d_status;
};

// The mixed solve (peec_gb300_complex_solve_mixed_device when cap is NULL;
// its graph form, enqueued on the calling thread's stream, otherwise).
int mixed_solve_impl(const Complex *d_Z, size_t n, const Complex *d_b, Complex *d_x, size_t nrhs, double tol,
                     int max_iter, double *backward_error, int *iterations, const MixedCapture *cap);

}  // namespace peec
