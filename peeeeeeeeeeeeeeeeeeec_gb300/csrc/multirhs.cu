// Many right-hand sides at once for the mixed-precision solve (hundreds of
// plane waves on one system): blocked triangular solves whose off-diagonal
// work is a GEMM, and the refinement residual in GEMM form that reads Z once
// per tile of right-hand sides instead of once per right-hand side, in
// double-float arithmetic on the FP32 pipes (FP64-equivalent to ~48 bits).
//
// Reference: complex_lu_solve_multiple (complex_lu.c:786-840) solves each
// right-hand side by itself (x = b / row_scale, pivots, forward, backward,
// / column_scale); here the same steps run for all of them together on the
// FP32 factor, and the FP64 iterative refinement around them checks each
// right-hand side's componentwise backward error (harmonic.c:899-1040).
//
// Layouts: right-hand sides and solutions are stored one after another
// ([nrhs][n], FP64 complex); the FP32 working block Y is unknown-major
// ([n][nrhs]) so that a row of it is one coalesced read for the GEMM and one
// value per thread in the diagonal-block solves.
#include <math.h>

#include "common.cuh"

namespace peec {
namespace mrhs {

struct c64 {
    double re, im;
};
struct c32 {
    float re, im;
};

static const int kDB = 64;  // rows of a diagonal block

// Y[i][q] = r[q][perm[i]] / rs[perm[i]] in FP32, through a 32 x 32 tile of
// shared memory (coalesced on both sides).
__global__ void __launch_bounds__(256) k_permute_in(const c64 *r, const int *perm, const double *rs, int n, int nrhs,
                                                    c32 *Y) {
    __shared__ c32 t[32][33];
    const int i0 = blockIdx.x * 32, q0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    for (int k = ty; k < 32; k += 8) {
        const int q = q0 + k, i = i0 + tx;
        c32 v = {0.0f, 0.0f};
        if (q < nrhs && i < n) {
            const int src = perm[i];
            const c64 z = r[(size_t)q * n + src];
            const double s = rs[src];
            v = c32{(float)(z.re / s), (float)(z.im / s)};
        }
        t[k][tx] = v;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int i = i0 + k, q = q0 + tx;
        if (i < n && q < nrhs) Y[(size_t)i * nrhs + q] = t[tx][k];
    }
}

// x[q][i] += Y[i][q] / cs[i] (FP64 accumulation), absx[q][i] = |x| in FP32.
__global__ void __launch_bounds__(256) k_update_out(c64 *x, const c32 *Y, const double *cs, int n, int nrhs,
                                                    float *absx) {
    __shared__ c32 t[32][33];
    const int i0 = blockIdx.x * 32, q0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int k = ty; k < 32; k += 8) {
        const int i = i0 + k, q = q0 + tx;
        t[k][tx] = (i < n && q < nrhs) ? Y[(size_t)i * nrhs + q] : c32{0.0f, 0.0f};
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int q = q0 + k, i = i0 + tx;
        if (q < nrhs && i < n) {
            const c32 y = t[tx][k];
            const double s = cs[i];
            c64 v = x[(size_t)q * n + i];
            v.re += (double)y.re / s;
            v.im += (double)y.im / s;
            x[(size_t)q * n + i] = v;
            const float ar = fminf(fabsf((float)v.re), 1e19f), ai = fminf(fabsf((float)v.im), 1e19f);
            absx[(size_t)q * n + i] = sqrtf(fmaf(ar, ar, ai * ai));
        }
    }
}

// The diagonal block rows r0..r0 + nrow - 1 of the packed factor solved for
// every right-hand side, one warp per right-hand side (lane l holds rows l
// and l + 32): unit lower (LOWER) forward substitution, or upper backward
// substitution with the division by u_ii; the block is staged in shared
// memory (rows past nrow act as identity), 8 right-hand sides per CTA.
__device__ __forceinline__ c32 shfl_c32(c32 v, int src) {
    return c32{__shfl_sync(0xffffffffu, v.re, src), __shfl_sync(0xffffffffu, v.im, src)};
}
__device__ __forceinline__ c32 msub_c32(c32 c, c32 a, c32 b) {  // c - a b
    c.re = fmaf(-a.re, b.re, c.re);
    c.re = fmaf(a.im, b.im, c.re);
    c.im = fmaf(-a.re, b.im, c.im);
    c.im = fmaf(-a.im, b.re, c.im);
    return c;
}

template <bool LOWER>
__global__ void __launch_bounds__(256) k_trsm_diag(const c32 *lu, int n, int r0, int nrow, c32 *Y, int nrhs) {
    __shared__ c32 B[kDB][kDB + 1];
    for (int t = threadIdx.x; t < kDB * kDB; t += blockDim.x) {
        const int i = t / kDB, j = t % kDB;
        c32 v = {i == j ? 1.0f : 0.0f, 0.0f};
        if (i < nrow && j < nrow) v = lu[(size_t)(r0 + i) * n + r0 + j];
        B[i][j] = v;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (q >= nrhs) return;
    c32 v0 = lane < nrow ? Y[(size_t)(r0 + lane) * nrhs + q] : c32{0.0f, 0.0f};
    c32 v1 = lane + 32 < nrow ? Y[(size_t)(r0 + lane + 32) * nrhs + q] : c32{0.0f, 0.0f};
    if (LOWER) {
        for (int j = 0; j < kDB - 1; ++j) {
            const c32 xj = shfl_c32(j < 32 ? v0 : v1, j & 31);
            if (lane > j) v0 = msub_c32(v0, B[lane][j], xj);
            if (lane + 32 > j) v1 = msub_c32(v1, B[lane + 32][j], xj);
        }
    } else {
        for (int j = kDB - 1; j >= 0; --j) {
            const c32 yj = shfl_c32(j < 32 ? v0 : v1, j & 31);
            const c32 d = B[j][j];
            const float den = d.re * d.re + d.im * d.im;
            const c32 xj = {(yj.re * d.re + yj.im * d.im) / den, (yj.im * d.re - yj.re * d.im) / den};
            if (lane < j) v0 = msub_c32(v0, B[lane][j], xj);
            if (lane + 32 < j) v1 = msub_c32(v1, B[lane + 32][j], xj);
            if (lane == (j & 31)) {
                if (j < 32)
                    v0 = xj;
                else
                    v1 = xj;
            }
        }
    }
    if (lane < nrow) Y[(size_t)(r0 + lane) * nrhs + q] = v0;
    if (lane + 32 < nrow) Y[(size_t)(r0 + lane + 32) * nrhs + q] = v1;
}

// C[i][q] -= sum_k A[i][k] Bm[k][q], complex FP32 on the CUDA cores:
// M x NC output, K <= 64; A rows with leading dimension lda, Bm and C with
// leading dimension ldb.  64 x 64 output tiles, 256 threads, 4 x 4 outputs
// per thread, K in chunks of 16 staged in shared memory.
__global__ void __launch_bounds__(256) k_cgemm_sub(const c32 *A, int lda, const c32 *Bm, c32 *C, int ldb, int M,
                                                   int NC, int K) {
    __shared__ c32 As[16][64 + 1];
    __shared__ c32 Bs[16][64];
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const int tr = threadIdx.x >> 4, tc = threadIdx.x & 15;  // 16 x 16 threads
    c32 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = c32{0.0f, 0.0f};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int t = threadIdx.x; t < 64 * 16; t += 256) {
            const int r = t >> 4, k = t & 15;  // A: row r, column k
            As[k][r] = (m0 + r < M && k0 + k < K) ? A[(size_t)(m0 + r) * lda + k0 + k] : c32{0.0f, 0.0f};
            const int kk = t >> 6, c = t & 63;  // Bm: row kk, column c
            Bs[kk][c] = (k0 + kk < K && n0 + c < NC) ? Bm[(size_t)(k0 + kk) * ldb + n0 + c] : c32{0.0f, 0.0f};
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            c32 a[4], b[4];
#pragma unroll
            for (int x = 0; x < 4; ++x) a[x] = As[k][tr + 16 * x];
#pragma unroll
            for (int y = 0; y < 4; ++y) b[y] = Bs[k][tc + 16 * y];
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) {
                    acc[x][y].re = fmaf(a[x].re, b[y].re, acc[x][y].re);
                    acc[x][y].re = fmaf(-a[x].im, b[y].im, acc[x][y].re);
                    acc[x][y].im = fmaf(a[x].re, b[y].im, acc[x][y].im);
                    acc[x][y].im = fmaf(a[x].im, b[y].re, acc[x][y].im);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int i = m0 + tr + 16 * x;
        if (i >= M) continue;
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const int q = n0 + tc + 16 * y;
            if (q >= NC) continue;
            c32 &c = C[(size_t)i * ldb + q];
            c.re -= acc[x][y].re;
            c.im -= acc[x][y].im;
        }
    }
}

// ---- real FP64: the inverse of an LU-factored matrix (transient system) ----

// The real diagonal block solved for every right-hand side, one warp per
// right-hand side (as k_trsm_diag).
template <bool LOWER>
__global__ void __launch_bounds__(256) k_trsm_diag_d(const double *lu, int n, int r0, int nrow, double *Y,
                                                     int nrhs) {
    __shared__ double B[kDB][kDB + 1];
    for (int t = threadIdx.x; t < kDB * kDB; t += blockDim.x) {
        const int i = t / kDB, j = t % kDB;
        double v = i == j ? 1.0 : 0.0;
        if (i < nrow && j < nrow) v = lu[(size_t)(r0 + i) * n + r0 + j];
        B[i][j] = v;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (q >= nrhs) return;
    double v0 = lane < nrow ? Y[(size_t)(r0 + lane) * nrhs + q] : 0.0;
    double v1 = lane + 32 < nrow ? Y[(size_t)(r0 + lane + 32) * nrhs + q] : 0.0;
    if (LOWER) {
        for (int j = 0; j < kDB - 1; ++j) {
            const double xj = __shfl_sync(0xffffffffu, j < 32 ? v0 : v1, j & 31);
            if (lane > j) v0 = fma(-B[lane][j], xj, v0);
            if (lane + 32 > j) v1 = fma(-B[lane + 32][j], xj, v1);
        }
    } else {
        for (int j = kDB - 1; j >= 0; --j) {
            const double xj = __shfl_sync(0xffffffffu, j < 32 ? v0 : v1, j & 31) / B[j][j];
            if (lane < j) v0 = fma(-B[lane][j], xj, v0);
            if (lane + 32 < j) v1 = fma(-B[lane + 32][j], xj, v1);
            if (lane == (j & 31)) {
                if (j < 32)
                    v0 = xj;
                else
                    v1 = xj;
            }
        }
    }
    if (lane < nrow) Y[(size_t)(r0 + lane) * nrhs + q] = v0;
    if (lane + 32 < nrow) Y[(size_t)(r0 + lane + 32) * nrhs + q] = v1;
}

// C[i][q] -= sum_k A[i][k] Bm[k][q] in FP64 (as k_cgemm_sub).
__global__ void __launch_bounds__(256) k_dgemm_sub(const double *A, int lda, const double *Bm, double *C, int ldb,
                                                   int M, int NC, int K) {
    __shared__ double As[16][64 + 1];
    __shared__ double Bs[16][64];
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const int tr = threadIdx.x >> 4, tc = threadIdx.x & 15;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int t = threadIdx.x; t < 64 * 16; t += 256) {
            const int r = t >> 4, k = t & 15;
            As[k][r] = (m0 + r < M && k0 + k < K) ? A[(size_t)(m0 + r) * lda + k0 + k] : 0.0;
            const int kk = t >> 6, c = t & 63;
            Bs[kk][c] = (k0 + kk < K && n0 + c < NC) ? Bm[(size_t)(k0 + kk) * ldb + n0 + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            double a[4], b[4];
#pragma unroll
            for (int x = 0; x < 4; ++x) a[x] = As[k][tr + 16 * x];
#pragma unroll
            for (int y = 0; y < 4; ++y) b[y] = Bs[k][tc + 16 * y];
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int i = m0 + tr + 16 * x;
        if (i >= M) continue;
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const int q = n0 + tc + 16 * y;
            if (q < NC) C[(size_t)i * ldb + q] -= acc[x][y];
        }
    }
}

// Y[i][q] = 1 where perm[i] == q, else 0: the permuted identity P I.
__global__ void k_permuted_identity(const int *perm, int n, double *Y) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)n * n) return;
    const int i = (int)(t / n), q = (int)(t % n);
    Y[t] = perm[i] == q ? 1.0 : 0.0;
}

// ---- double-float residual: the same product on the FP32 pipes ----
// A double-float value is an unevaluated sum hi + lo of two floats (~48
// significant bits).  Products use the exact FMA product of the high parts
// plus the cross terms; sums use the error-free two-sum of the high parts
// (Dekker 1971, Knuth TAOCP 4.2.2).  On GB300 the FP32 pipe issues ~60x the
// FP64 pipe's rate, so ~15 FP32 operations per real multiply-add still run
// ~4x faster than one FP64 FMA.

struct df {
    float h, l;
};

__device__ __forceinline__ df df_split(double v) {
    const float h = (float)v;
    return df{h, (float)(v - (double)h)};
}

// s + a b
__device__ __forceinline__ df df_mac(df s, df a, df b) {
    const float ph = a.h * b.h;
    float pl = fmaf(a.h, b.h, -ph);
    pl = fmaf(a.h, b.l, pl);
    pl = fmaf(a.l, b.h, pl);
    const float t = s.h + ph;
    const float bb = t - s.h;
    float e = (s.h - (t - bb)) + (ph - bb);
    e += s.l + pl;
    const float hh = t + e;
    return df{hh, e - (hh - t)};
}

struct df4 {
    df re, im;
};

// R[q][i] = B[q][i] - sum_j Z[i][j] X[q][j] for all right-hand sides, with
// the componentwise backward error |R_qi| / (sum_j |Z_ij||X_qj| + |B_qi|)
// (the denominator from FP32 magnitudes absZ, absx) max-reduced into *be as
// IEEE bits.  64 rows x 32 right-hand sides per CTA, 256 threads of 4 rows
// x 2 right-hand sides, K in chunks of 16 in shared memory: Z is read once
// per 32 right-hand sides.  The tiles of Z and X are split into float pairs
// as they are staged (each split serves 32 right-hand sides or 64 rows),
// the 8 complex accumulators of a thread are double-float, and the residual
// is formed in FP64 from them at the end.
__global__ void __launch_bounds__(256) k_residual_gemm_df(const c64 *Z, const float *absZ, const c64 *X,
                                                          const float *absx, const c64 *B, int n, int nrhs, c64 *R,
                                                          unsigned long long *be) {
    __shared__ df4 Zs[16][64 + 1];
    __shared__ float Za[16][64 + 1];
    __shared__ df4 Xs[16][32 + 1];
    __shared__ float Xa[16][32 + 1];
    const int i0 = blockIdx.y * 64, q0 = blockIdx.x * 32;
    const int tr = threadIdx.x >> 4, tq = threadIdx.x & 15;
    df4 acc[4][2];
    float den[4][2];
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
            acc[x][y] = df4{{0.0f, 0.0f}, {0.0f, 0.0f}};
            den[x][y] = 0.0f;
        }
    for (int j0 = 0; j0 < n; j0 += 16) {
        for (int t = threadIdx.x; t < 64 * 16; t += 256) {
            const int r = t >> 4, k = t & 15;
            const bool ok = i0 + r < n && j0 + k < n;
            const c64 z = ok ? Z[(size_t)(i0 + r) * n + j0 + k] : c64{0.0, 0.0};
            Zs[k][r] = df4{df_split(z.re), df_split(z.im)};
            Za[k][r] = ok ? absZ[(size_t)(i0 + r) * n + j0 + k] : 0.0f;
        }
        for (int t = threadIdx.x; t < 32 * 16; t += 256) {
            const int c = t >> 4, k = t & 15;
            const bool ok = q0 + c < nrhs && j0 + k < n;
            const c64 v = ok ? X[(size_t)(q0 + c) * n + j0 + k] : c64{0.0, 0.0};
            Xs[k][c] = df4{df_split(v.re), df_split(v.im)};
            Xa[k][c] = ok ? absx[(size_t)(q0 + c) * n + j0 + k] : 0.0f;
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < 16; ++k) {
            df4 z[4], v[2];
            float za[4], va[2];
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                z[x] = Zs[k][tr + 16 * x];
                za[x] = Za[k][tr + 16 * x];
            }
#pragma unroll
            for (int y = 0; y < 2; ++y) {
                v[y] = Xs[k][tq + 16 * y];
                va[y] = Xa[k][tq + 16 * y];
            }
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 2; ++y) {
                    const df nzi = {-z[x].im.h, -z[x].im.l};
                    acc[x][y].re = df_mac(acc[x][y].re, z[x].re, v[y].re);
                    acc[x][y].re = df_mac(acc[x][y].re, nzi, v[y].im);
                    acc[x][y].im = df_mac(acc[x][y].im, z[x].re, v[y].im);
                    acc[x][y].im = df_mac(acc[x][y].im, z[x].im, v[y].re);
                    den[x][y] = fmaf(za[x], va[y], den[x][y]);
                }
        }
        __syncthreads();
    }
    double worst = 0.0;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int i = i0 + tr + 16 * x;
        if (i >= n) continue;
#pragma unroll
        for (int y = 0; y < 2; ++y) {
            const int q = q0 + tq + 16 * y;
            if (q >= nrhs) continue;
            const c64 b = B[(size_t)q * n + i];
            const double yre = (double)acc[x][y].re.h + (double)acc[x][y].re.l;
            const double yim = (double)acc[x][y].im.h + (double)acc[x][y].im.l;
            const c64 r = c64{b.re - yre, b.im - yim};
            R[(size_t)q * n + i] = r;
            const double res = sqrt(fma(r.re, r.re, r.im * r.im));
            const double babs = hypot(b.re, b.im);
            const double d = (double)den[x][y] + babs;
            double eta = d > 0.0 ? res / d : res;
            if (!isfinite(eta)) eta = INFINITY;
            worst = fmax(worst, eta);
        }
    }
    atomicMax(be, (unsigned long long)__double_as_longlong(worst));
}

}  // namespace mrhs

// The inverse of a matrix from its packed FP64 LU factor (unit L, U, row
// permutation perm as the solves use it): X = U^-1 L^-1 P, i.e. the blocked
// forward and backward substitution of the permuted identity, all n columns
// at once, into Minv (n x n row-major).  About 2 n^3 FP64 flops.
bool inverse_from_lu_real(const double *lu, const int *perm, int n, double *Minv) {
    using namespace mrhs;
    PEEC_LAUNCH(k_permuted_identity, (unsigned)(((size_t)n * n + 255) / 256), 256, 0, perm, n, Minv);
    const int nb = (n + kDB - 1) / kDB;
    const unsigned dgrid = (unsigned)((n + 7) / 8);
    for (int blk = 0; blk < nb; ++blk) {
        const int r0 = blk * kDB, nrow = min(kDB, n - r0), r1 = r0 + nrow;
        PEEC_LAUNCH(k_trsm_diag_d<true>, dgrid, 256, 0, lu, n, r0, nrow, Minv, n);
        if (r1 < n)
            PEEC_LAUNCH(k_dgemm_sub, dim3((n + 63) / 64, (n - r1 + 63) / 64), 256, 0, lu + (size_t)r1 * n + r0, n,
                        Minv + (size_t)r0 * n, Minv + (size_t)r1 * n, n, n - r1, n, nrow);
    }
    for (int blk = nb - 1; blk >= 0; --blk) {
        const int r0 = blk * kDB, nrow = min(kDB, n - r0);
        PEEC_LAUNCH(k_trsm_diag_d<false>, dgrid, 256, 0, lu, n, r0, nrow, Minv, n);
        if (r0 > 0)
            PEEC_LAUNCH(k_dgemm_sub, dim3((n + 63) / 64, (r0 + 63) / 64), 256, 0, lu + r0, n, Minv + (size_t)r0 * n,
                        Minv, n, r0, n, nrow);
    }
    return launch_ok("inverse from the LU factor");
}

// One correction of the many-right-hand-side refinement, all on the
// calling thread's stream: Y = P D_r^-1 r (FP32, [n][nrhs]); forward and
// backward block substitution on the FP32 factor lu (diagonal blocks per
// right-hand side, the rest as GEMMs); x += D_c^-1 Y; r = b - Z x (FP64) and
// the backward error into *be (IEEE bits; the caller zeroes it).
bool mrhs_sweep(const void *Z, const float *absZ, const void *lu, const int *perm, const double *rs,
                const double *cs, int n, int nrhs, const void *b, void *x, void *r, void *Y, float *absx,
                unsigned long long *be) {
    using namespace mrhs;
    const c32 *F = (const c32 *)lu;
    c32 *Yt = (c32 *)Y;
    const dim3 tgrid((n + 31) / 32, (nrhs + 31) / 32);
    PEEC_LAUNCH(k_permute_in, tgrid, 256, 0, (const c64 *)r, perm, rs, n, nrhs, Yt);
    const int nb = (n + kDB - 1) / kDB;
    const unsigned dgrid = (unsigned)((nrhs + 7) / 8);
    for (int blk = 0; blk < nb; ++blk) {  // forward: unit lower
        const int r0 = blk * kDB, nrow = min(kDB, n - r0), r1 = r0 + nrow;
        PEEC_LAUNCH(k_trsm_diag<true>, dgrid, 256, 0, F, n, r0, nrow, Yt, nrhs);
        if (r1 < n)
            PEEC_LAUNCH(k_cgemm_sub, dim3((nrhs + 63) / 64, (n - r1 + 63) / 64), 256, 0, F + (size_t)r1 * n + r0, n,
                        Yt + (size_t)r0 * nrhs, Yt + (size_t)r1 * nrhs, nrhs, n - r1, nrhs, nrow);
    }
    for (int blk = nb - 1; blk >= 0; --blk) {  // backward: upper
        const int r0 = blk * kDB, nrow = min(kDB, n - r0);
        PEEC_LAUNCH(k_trsm_diag<false>, dgrid, 256, 0, F, n, r0, nrow, Yt, nrhs);
        if (r0 > 0)
            PEEC_LAUNCH(k_cgemm_sub, dim3((nrhs + 63) / 64, (r0 + 63) / 64), 256, 0, F + r0, n,
                        Yt + (size_t)r0 * nrhs, Yt, nrhs, r0, nrhs, nrow);
    }
    PEEC_LAUNCH(k_update_out, tgrid, 256, 0, (c64 *)x, Yt, cs, n, nrhs, absx);
    PEEC_LAUNCH(k_residual_gemm_df, dim3((nrhs + 31) / 32, (n + 63) / 64), 256, 0, (const c64 *)Z, absZ,
                (const c64 *)x, absx, (const c64 *)b, n, nrhs, (c64 *)r, be);
    return launch_ok("many-right-hand-side sweep");
}

}  // namespace peec
