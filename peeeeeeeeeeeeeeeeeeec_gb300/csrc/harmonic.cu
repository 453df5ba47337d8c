// Device-resident harmonic system around the hot path: the MNA fill that
// consumes Lp and P, a plane-wave right-hand side, and the componentwise
// backward error that gates every solve.
//
// Reference (paths inside the reference project):
//   src/solver/harmonic.c:175-372    harmonic_build_system
//       Z = [ R + j w L     A    ]      A[e,a] = -1, A[e,b] = +1 (incidence.c:34-110)
//           [ -P A^T      j w I  ]      (P A^T)[i,e] = P[i,b] - P[i,a] (incidence.c:417-592)
//   src/solver/harmonic.c:436-552    harmonic_build_rhs: [-U_e ; P I_s]
//   src/physics/scattering.c:263-336 U_e = (E(r_c) . l) sinc(k_hat.l k0 / 2)
//   src/physics/incident_field.c:754-830  E(r) = E0 exp(-j k0 k_hat.r)
//   src/solver/harmonic.c:720-1080   backward error max_i |r_i| / (sum_j |Z_ij||x_j| + |b_i|)
// All byte-bound: one pass over Z per kernel.
#include <math.h>

#include "../../include/complex_matrix.h"
#include "../../include/peec_gb300.h"
#include "common.cuh"

namespace peec {

struct cpx {
    double re, im;
};

// One thread per entry of row-block rows; coalesced 16-byte stores.
__global__ void k_harmonic_fill(const double *L, const double *P, const int *edges, const double *R, int ne, int nv,
                                double omega, const double *omega_dev, cpx *Z) {
    if (omega_dev) omega = *omega_dev;  // the batched sweep's graph: the frequency lives in device memory
    const long long n = (long long)ne + nv;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n * n;
         t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t / n), j = (int)(t % n);
        cpx z = {0.0, 0.0};
        if (i < ne) {
            if (j < ne) {
                z.re = (i == j && R) ? R[i] : 0.0;
                z.im = omega * L[(size_t)i * ne + j];
            } else {
                int k = j - ne;
                z.re = (k == edges[2 * i]) ? -1.0 : (k == edges[2 * i + 1]) ? 1.0 : 0.0;
            }
        } else {
            int r = i - ne;
            if (j < ne) {
                int a = edges[2 * j], b = edges[2 * j + 1];
                const double *prow = P + (size_t)r * nv;
                z.re = -(prow[b] - prow[a]);
            } else if (j - ne == r) {
                z.im = omega;
            }
        }
        Z[t] = z;
    }
}

// The same system from retarded (complex) Lp and P: j w (Lr + j Li) and
// -(P A^T) with complex P.
__global__ void k_harmonic_fill_complex(const cpx *L, const cpx *P, const int *edges, const double *R, int ne, int nv,
                                        double omega, cpx *Z) {
    const long long n = (long long)ne + nv;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n * n;
         t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t / n), j = (int)(t % n);
        cpx z = {0.0, 0.0};
        if (i < ne) {
            if (j < ne) {
                cpx l = L[(size_t)i * ne + j];
                z.re = ((i == j && R) ? R[i] : 0.0) - omega * l.im;
                z.im = omega * l.re;
            } else {
                int k = j - ne;
                z.re = (k == edges[2 * i]) ? -1.0 : (k == edges[2 * i + 1]) ? 1.0 : 0.0;
            }
        } else {
            int r = i - ne;
            if (j < ne) {
                int a = edges[2 * j], b = edges[2 * j + 1];
                const cpx *prow = P + (size_t)r * nv;
                z.re = -(prow[b].re - prow[a].re);
                z.im = -(prow[b].im - prow[a].im);
            } else if (j - ne == r) {
                z.im = omega;
            }
        }
        Z[t] = z;
    }
}

// U_e for a plane wave E(r) = e_hat exp(-j k0 k_hat.r) in the operation
// order of the reference (incident_field.c:754-830, scattering.c:140-336):
// E_k = (e_k cos g, e_k sin g) with g = -k0 (k_hat.r_c) + 0, projected on
// the edge vector term by term, times sinc(k0 (k_hat.l) / 2) with the
// series 1 - x^2/6 + x^4/120 below |x| = 1e-4; the right-hand side is
// [-U_e ; 0].  The library is built without FMA contraction, so only the
// device sin / cos can differ from the host's (by an ulp).
__device__ __forceinline__ cpx plane_wave_edge(const double *c, const double *l, double kx, double ky, double kz,
                                               double ex, double ey, double ez, double k0) {
    double kr = kx * c[0] + ky * c[1] + kz * c[2];
    double g = -k0 * kr + 0.0;
    double s, co;
    sincos(g, &s, &co);
    double ure = (ex * co) * l[0] + (ey * co) * l[1] + (ez * co) * l[2];
    double uim = (ex * s) * l[0] + (ey * s) * l[1] + (ez * s) * l[2];
    double x = 0.5 * (k0 * (kx * l[0] + ky * l[1] + kz * l[2]));
    double f;
    if (fabs(x) < 1.0e-4) {
        double x2 = x * x;
        f = 1.0 - x2 / 6.0 + (x2 * x2) / 120.0;
    } else {
        f = sin(x) / x;
    }
    return cpx{-(ure * f), -(uim * f)};
}

__global__ void k_plane_wave_rhs(const double *centers, const double *vectors, int ne, int nv, double kx, double ky,
                                 double kz, double ex, double ey, double ez, double k0, cpx *rhs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ne + nv) return;
    rhs[i] = i >= ne ? cpx{0.0, 0.0}
                     : plane_wave_edge(centers + 3 * i, vectors + 3 * i, kx, ky, kz, ex, ey, ez, k0);
}

// nrhs waves at once (directions and polarisations in device memory, k0
// from *k0_dev when set): rhs[q][i].
__global__ void k_plane_waves(const double *centers, const double *vectors, int ne, int nv, int nrhs,
                              const double *k_hat, const double *e_hat, double k0, const double *k0_dev, cpx *rhs) {
    const long long n = (long long)ne + nv;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n * nrhs) return;
    if (k0_dev) k0 = *k0_dev;
    const int q = (int)(t / n), i = (int)(t % n);
    const double *kq = k_hat + 3 * q, *eq = e_hat + 3 * q;
    rhs[t] = i >= ne ? cpx{0.0, 0.0}
                     : plane_wave_edge(centers + 3 * i, vectors + 3 * i, kq[0], kq[1], kq[2], eq[0], eq[1], eq[2], k0);
}

// |z| in FP32 for the denominator sum |Z||x| + |b| of the backward error (a
// gate, not a result: FP32 rounding moves eta by ~1e-7 of itself).  Parts
// are clamped to 1e19 so the square cannot overflow; clamping and underflow
// can only shrink the denominator, i.e. overstate eta.
__device__ __forceinline__ float abs_f32_fast(cpx z) {
    float ar = fminf(fabsf((float)z.re), 1e19f), ai = fminf(fabsf((float)z.im), 1e19f);
    return sqrtf(fmaf(ar, ar, ai * ai));
}

__global__ void k_abs_vector(const cpx *x, size_t count, float *out) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t < count) out[t] = abs_f32_fast(x[t]);
}

// Componentwise backward error, one warp per row; results as IEEE bits
// (non-negative) max-reduced: out[0] = backward error, out[1] = max |r_i|,
// out[2] = max |b_i|.  The residual is FP64, the denominator FP32.
__global__ void k_backward_error(const cpx *Z, const cpx *x, const float *absx, const cpx *b, int n, int nrhs,
                                 unsigned long long *out) {
    long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= (long long)n * nrhs) return;
    int rr = (int)(warp / n), i = (int)(warp % n);
    const cpx *row = Z + (size_t)i * n;
    const cpx *xr = x + (size_t)rr * n;
    const float *ax = absx + (size_t)rr * n;
    double yr = 0.0, yi = 0.0;
    float den = 0.0f;
    for (int j = lane; j < n; j += 32) {
        cpx z = row[j], v = xr[j];
        yr = fma(z.re, v.re, yr);
        yr = fma(-z.im, v.im, yr);
        yi = fma(z.re, v.im, yi);
        yi = fma(z.im, v.re, yi);
        den = fmaf(abs_f32_fast(z), ax[j], den);
    }
    yr = warp_sum(yr);
    yi = warp_sum(yi);
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) den += __shfl_xor_sync(0xffffffffu, den, m);
    if (lane == 0) {
        cpx bi = b[(size_t)rr * n + i];
        double res = hypot(yr - bi.re, yi - bi.im);
        double babs = hypot_cr(bi.re, bi.im);
        double d = (double)den + babs;
        double eta = d > 0.0 ? res / d : res;
        if (!isfinite(eta)) eta = INFINITY;
        atomicMax(out + 0, (unsigned long long)__double_as_longlong(eta));
        atomicMax(out + 1, (unsigned long long)__double_as_longlong(isfinite(res) ? res : INFINITY));
        atomicMax(out + 2, (unsigned long long)__double_as_longlong(babs));
    }
}

// Launchers for the batched sweep (sweep.cu): omega / k0 read from device
// memory by the kernels, so that a recorded graph serves every frequency.
bool launch_harmonic_fill_dev(const double *L, const double *P, const int *edges, const double *R, int ne, int nv,
                              const double *omega_dev, void *Z) {
    long long n = (long long)ne + nv, total = n * n;
    int grid = (int)((total + 255) / 256 < 152LL * 32 ? (total + 255) / 256 : 152LL * 32);
    PEEC_LAUNCH(k_harmonic_fill, grid, 256, 0, L, P, edges, R, ne, nv, 0.0, omega_dev, (cpx *)Z);
    return launch_ok("harmonic fill");
}

bool launch_plane_waves_dev(const double *centers, const double *vectors, int ne, int nv, int nrhs,
                            const double *d_k_hat, const double *d_e_hat, const double *k0_dev, void *rhs) {
    long long total = ((long long)ne + nv) * nrhs;
    PEEC_LAUNCH(k_plane_waves, (unsigned)((total + 255) / 256), 256, 0, centers, vectors, ne, nv, nrhs, d_k_hat,
                d_e_hat, 0.0, k0_dev, (cpx *)rhs);
    return launch_ok("plane waves");
}

}  // namespace peec

using namespace peec;

extern "C" {

int peec_gb300_harmonic_build_device(const double *d_L, const double *d_P, const int *d_edges,
                                     const double *d_R, size_t n_edges, size_t n_nodes, double frequency,
                                     Complex *d_Z) {
    if (!d_L || !d_P || !d_edges || !d_Z || n_edges == 0 || n_nodes == 0 || !isfinite(frequency) ||
        frequency <= 0.0)
        return -1;
    double omega = 2.0 * M_PI * frequency;
    long long n = (long long)(n_edges + n_nodes);
    long long total = n * n;
    int grid = (int)((total + 255) / 256 < 152LL * 32 ? (total + 255) / 256 : 152LL * 32);
    PEEC_LAUNCH(k_harmonic_fill, grid, 256, 0, d_L, d_P, d_edges, d_R, (int)n_edges, (int)n_nodes, omega,
                (const double *)nullptr, (cpx *)d_Z);
    return launch_ok("harmonic fill") ? 0 : -1;
}

int peec_gb300_harmonic_build_retarded_device(const Complex *d_L, const Complex *d_P, const int *d_edges,
                                              const double *d_R, size_t n_edges, size_t n_nodes, double frequency,
                                              Complex *d_Z) {
    if (!d_L || !d_P || !d_edges || !d_Z || n_edges == 0 || n_nodes == 0 || !isfinite(frequency) ||
        frequency <= 0.0)
        return -1;
    double omega = 2.0 * M_PI * frequency;
    long long n = (long long)(n_edges + n_nodes);
    long long total = n * n;
    int grid = (int)((total + 255) / 256 < 152LL * 32 ? (total + 255) / 256 : 152LL * 32);
    PEEC_LAUNCH(k_harmonic_fill_complex, grid, 256, 0, (const cpx *)d_L, (const cpx *)d_P, d_edges, d_R,
                (int)n_edges, (int)n_nodes, omega, (cpx *)d_Z);
    return launch_ok("retarded harmonic fill") ? 0 : -1;
}

int peec_gb300_plane_wave_rhs_device(const double *d_edge_centers, const double *d_edge_vectors, size_t n_edges,
                                     size_t n_nodes, const double k_hat[3], const double e_hat[3],
                                     double wave_number, Complex *d_rhs) {
    if (!d_edge_centers || !d_edge_vectors || !k_hat || !e_hat || !d_rhs) return -1;
    int n = (int)(n_edges + n_nodes);
    PEEC_LAUNCH(k_plane_wave_rhs, (n + 255) / 256, 256, 0, d_edge_centers, d_edge_vectors, (int)n_edges,
                (int)n_nodes, k_hat[0], k_hat[1], k_hat[2], e_hat[0], e_hat[1], e_hat[2], wave_number, (cpx *)d_rhs);
    return launch_ok("plane-wave rhs") ? 0 : -1;
}

int peec_gb300_backward_error_device(const Complex *d_Z, size_t n, const Complex *d_x, const Complex *d_b,
                                     size_t nrhs, double out[3]) {
    if (!d_Z || !d_x || !d_b || !out || n == 0 || nrhs == 0) return -1;
    DBuf<unsigned long long> acc(3);
    DBuf<float> absx(n * nrhs);
    if (!acc.p || !absx.p) return -1;
    cudaMemsetAsync(acc.p, 0, 3 * sizeof(unsigned long long), stream());
    PEEC_LAUNCH(k_abs_vector, (unsigned)((n * nrhs + 255) / 256), 256, 0, (const cpx *)d_x, n * nrhs, absx.p);
    long long warps = (long long)n * nrhs;
    PEEC_LAUNCH(k_backward_error, (unsigned)((warps * 32 + 255) / 256), 256, 0, (const cpx *)d_Z, (const cpx *)d_x,
                absx.p, (const cpx *)d_b, (int)n, (int)nrhs, acc.p);
    unsigned long long h[3];
    cudaMemcpyAsync(h, acc.p, sizeof(h), cudaMemcpyDeviceToHost, stream());
    if (!sync("backward error")) return -1;
    for (int k = 0; k < 3; ++k) memcpy(&out[k], &h[k], sizeof(double));
    return 0;
}

}  // extern "C"
