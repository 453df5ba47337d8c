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

// x[q][i] += Y[i][q] / cs[i] (FP64 accumulation); xs[q][i] = x as float
// pairs (re.h, re.l, im.h, im.l) for the residual.
__global__ void __launch_bounds__(256) k_update_out(c64 *x, const c32 *Y, const double *cs, int n, int nrhs,
                                                    float4 *xs, const int *done) {
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
        if (q < nrhs && i < n && !done[q]) {
            const c32 y = t[tx][k];
            const double s = cs[i];
            c64 v = x[(size_t)q * n + i];
            v.re += (double)y.re / s;
            v.im += (double)y.im / s;
            x[(size_t)q * n + i] = v;
            const float rh = (float)v.re, ih = (float)v.im;
            xs[(size_t)q * n + i] = make_float4(rh, (float)(v.re - (double)rh), ih, (float)(v.im - (double)ih));
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
__global__ void __launch_bounds__(256) k_trsm_diag(const c32 *lu, int n, int r0, int nrow, c32 *Y, int nrhs,
                                                   const int *done) {
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
    if (q >= nrhs || done[q]) return;  // converged right-hand sides keep their solution
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
                                                   int NC, int K, const int *done) {
    __shared__ c32 As[16][64 + 1];
    __shared__ c32 Bs[16][64];
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    // a tile whose 64 right-hand sides have all converged has nothing to do
    const int qc = n0 + (threadIdx.x & 63);
    if (__syncthreads_and(qc >= NC || done[qc])) return;
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
// significant bits).  The products below take the exact FMA product of the
// high parts plus the two cross terms; the running sum of the high parts
// uses the error-free two-sum (Dekker 1971, Knuth TAOCP 4.2.2), and every
// low-order term (product errors, cross terms, two-sum errors) goes into a
// second FP32 accumulator that is folded in once, at the end.  On GB300 the
// FP32 pipe issues ~60x the FP64 pipe's rate, so the 12 FP32 operations of
// one real multiply-add still run ~5x faster than one FP64 FMA.
//
// The complex product uses Gauss's three real products: with s_z = re + im
// of Z and s_x = re + im of X (both double-float sums formed as the tiles
// are staged), T1 = sum re*re, T2 = sum im*im, T3 = sum s_z*s_x, and
// Re = T1 - T2, Im = T3 - T1 - T2 in FP64 at the end.  The error stays a
// few units of 2^-48 of sum |Z_ij||X_j|, the residual's own scale.

// Z as float pairs (re.h, re.l, im.h, im.l), once per solve: the residual
// tiles then stage no FP64 instructions.
__global__ void k_split_z(const c64 *Z, size_t count, float4 *Zs) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const c64 z = Z[t];
    const float rh = (float)z.re, ih = (float)z.im;
    Zs[t] = make_float4(rh, (float)(z.re - (double)rh), ih, (float)(z.im - (double)ih));
}

struct dacc {  // running sum: h (two-summed high parts) + l (low-order terms)
    float h, l;
};

// s += (ah + al)(bh + bl), dropping al bl
__device__ __forceinline__ void dmac(dacc &s, float ah, float al, float bh, float bl) {
    const float p = ah * bh;
    float e = fmaf(ah, bh, -p);
    const float t = s.h + p;
    const float bp = t - s.h;
    const float err = (s.h - (t - bp)) + (p - bp);
    s.h = t;
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
    s.l += e + err;
}

// (h, l) of a + b for two float pairs (two-sum of the high parts)
__device__ __forceinline__ float2 pair_sum(float ah, float al, float bh, float bl) {
    const float t = ah + bh;
    const float bp = t - ah;
    const float err = (ah - (t - bp)) + (bh - bp);
    const float l = err + al + bl;
    const float h = t + l;
    return make_float2(h, l - (h - t));
}

// R[q][i] = B[q][i] - sum_j Z[i][j] X[q][j] for all right-hand sides, with
// the componentwise backward error |R_qi| / (sum_j |Z_ij||X_qj| + |B_qi|)
// (the denominator in FP32 from the high parts) max-reduced into *be as
// IEEE bits.  Zs, Xs: Z and X as float pairs (k_split_z, k_update_out).
// 64 rows x 32 right-hand sides per CTA, 256 threads of 4 rows x 2
// right-hand sides, K in chunks of 16 in shared memory: Z is read once per
// 32 right-hand sides.  Each staged element holds its re and im pairs, its
// re + im pair and its FP32 magnitude, so the inner loop is FP32 only.
static const int kRK = 16;
struct RTile {  // rows padded by one element: the transposing stores are conflict-free
    float4 z[kRK][64 + 1];   // re.h, re.l, im.h, im.l
    float4 zs[kRK][64 + 1];  // (re + im).h, (re + im).l, |z|, 0
    float4 x[kRK][32 + 1];
    float4 xs[kRK][32 + 1];
};

__global__ void __launch_bounds__(256) k_residual_gemm_df(const float4 *Zs, const float4 *Xs, const c64 *B, int n,
                                                          int nrhs, c64 *R, unsigned long long *be,
                                                          unsigned long long *be_q, const int *done) {
    extern __shared__ __align__(16) unsigned char rsm[];
    RTile &S = *reinterpret_cast<RTile *>(rsm);
    const int i0 = blockIdx.y * 64, q0 = blockIdx.x * 32;
    // 32 converged right-hand sides: their residuals and errors stand
    const int qc = q0 + (threadIdx.x & 31);
    if (__syncthreads_and(qc >= nrhs || done[qc])) return;
    const int tr = threadIdx.x >> 4, tq = threadIdx.x & 15;
    dacc t1[4][2], t2[4][2], t3[4][2];
    float den[4][2];
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
            t1[x][y] = t2[x][y] = t3[x][y] = dacc{0.0f, 0.0f};
            den[x][y] = 0.0f;
        }
    for (int j0 = 0; j0 < n; j0 += kRK) {
        for (int t = threadIdx.x; t < 64 * kRK; t += 256) {
            const int r = t / kRK, k = t % kRK;
            float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (i0 + r < n && j0 + k < n) z = Zs[(size_t)(i0 + r) * n + j0 + k];
            const float2 sz = pair_sum(z.x, z.y, z.z, z.w);
            S.z[k][r] = z;
            S.zs[k][r] = make_float4(sz.x, sz.y, sqrtf(fmaf(z.x, z.x, z.z * z.z)), 0.0f);
        }
        for (int t = threadIdx.x; t < 32 * kRK; t += 256) {
            const int c = t / kRK, k = t % kRK;
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (q0 + c < nrhs && j0 + k < n) v = Xs[(size_t)(q0 + c) * n + j0 + k];
            const float2 sv = pair_sum(v.x, v.y, v.z, v.w);
            S.x[k][c] = v;
            S.xs[k][c] = make_float4(sv.x, sv.y, sqrtf(fmaf(v.x, v.x, v.z * v.z)), 0.0f);
        }
        __syncthreads();
#pragma unroll 2
        for (int k = 0; k < kRK; ++k) {
            float4 z[4], zs[4], v[2], vs[2];
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                z[x] = S.z[k][tr + 16 * x];
                zs[x] = S.zs[k][tr + 16 * x];
            }
#pragma unroll
            for (int y = 0; y < 2; ++y) {
                v[y] = S.x[k][tq + 16 * y];
                vs[y] = S.xs[k][tq + 16 * y];
            }
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 2; ++y) {
                    dmac(t1[x][y], z[x].x, z[x].y, v[y].x, v[y].y);
                    dmac(t2[x][y], z[x].z, z[x].w, v[y].z, v[y].w);
                    dmac(t3[x][y], zs[x].x, zs[x].y, vs[y].x, vs[y].y);
                    den[x][y] = fmaf(zs[x].z, vs[y].z, den[x][y]);
                }
        }
        __syncthreads();
    }
    double worst = 0.0, worst_q[2] = {0.0, 0.0};
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int i = i0 + tr + 16 * x;
        if (i >= n) continue;
#pragma unroll
        for (int y = 0; y < 2; ++y) {
            const int q = q0 + tq + 16 * y;
            if (q >= nrhs) continue;
            const c64 b = B[(size_t)q * n + i];
            const double a1 = (double)t1[x][y].h + (double)t1[x][y].l;
            const double a2 = (double)t2[x][y].h + (double)t2[x][y].l;
            const double a3 = (double)t3[x][y].h + (double)t3[x][y].l;
            const c64 r = c64{b.re - (a1 - a2), b.im - (a3 - a1 - a2)};
            R[(size_t)q * n + i] = r;
            const double res = sqrt(fma(r.re, r.re, r.im * r.im));
            const double babs = hypot(b.re, b.im);
            const double d = (double)den[x][y] + babs;
            double eta = d > 0.0 ? res / d : res;
            if (!isfinite(eta)) eta = INFINITY;
            worst = fmax(worst, eta);
            worst_q[y] = fmax(worst_q[y], eta);
        }
    }
    atomicMax(be, (unsigned long long)__double_as_longlong(worst));
#pragma unroll
    for (int y = 0; y < 2; ++y) {  // lanes l and l + 16 share a right-hand side
        const double w = fmax(worst_q[y], __shfl_xor_sync(0xffffffffu, worst_q[y], 16));
        const int q = q0 + tq + 16 * y;
        if ((threadIdx.x & 16) == 0 && q < nrhs) atomicMax(be_q + q, (unsigned long long)__double_as_longlong(w));
    }
}

// per right-hand side, before a sweep: the error maxima of the ones still
// refined start at zero; after it: the ones at the gate are marked done
__global__ void k_be_reset(unsigned long long *be_q, const int *done, int nrhs) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nrhs && !done[q]) be_q[q] = 0ull;
}
__global__ void k_mark_done(const unsigned long long *be_q, int *done, int nrhs, double tol) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nrhs && !done[q] && __longlong_as_double((long long)be_q[q]) <= tol) done[q] = 1;
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

// Z (count complex FP64 entries) as float pairs into Zs (16 bytes an entry),
// once per solve, for the residual of mrhs_sweep.
bool mrhs_split_z(const void *Z, size_t count, void *Zs) {
    using namespace mrhs;
    PEEC_LAUNCH(k_split_z, (unsigned)((count + 255) / 256), 256, 0, (const c64 *)Z, count, (float4 *)Zs);
    return launch_ok("many-right-hand-side split of Z");
}

// One correction of the many-right-hand-side refinement, all on the
// calling thread's stream: Y = P D_r^-1 r (FP32, [n][nrhs]); forward and
// backward block substitution on the FP32 factor lu (diagonal blocks per
// right-hand side, the rest as GEMMs); x += D_c^-1 Y (FP64) and its float
// pairs xs; r = b - Z x in double-float from the split Zs (mrhs_split_z) and
// the backward error into *be (IEEE bits; the caller zeroes it).  Right-
// hand sides refine until their own backward error reaches tol: done[q]
// (zeroed by the caller before the first sweep) then stops their updates,
// and tiles of done right-hand sides are skipped; be_q[q] holds each one's
// last backward error.
bool mrhs_sweep(const void *Zs, const void *lu, const int *perm, const double *rs, const double *cs, int n, int nrhs,
                const void *b, void *x, void *r, void *Y, void *xs, unsigned long long *be, unsigned long long *be_q,
                int *done, double tol) {
    using namespace mrhs;
    static const cudaError_t attr = cudaFuncSetAttribute(
        k_residual_gemm_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(RTile));
    if (!cuda_ok(attr, "residual GEMM shared memory attribute")) return false;
    const c32 *F = (const c32 *)lu;
    c32 *Yt = (c32 *)Y;
    const dim3 tgrid((n + 31) / 32, (nrhs + 31) / 32);
    const unsigned qgrid = (unsigned)((nrhs + 255) / 256);
    PEEC_LAUNCH(k_be_reset, qgrid, 256, 0, be_q, (const int *)done, nrhs);
    PEEC_LAUNCH(k_permute_in, tgrid, 256, 0, (const c64 *)r, perm, rs, n, nrhs, Yt);
    const int nb = (n + kDB - 1) / kDB;
    const unsigned dgrid = (unsigned)((nrhs + 7) / 8);
    for (int blk = 0; blk < nb; ++blk) {  // forward: unit lower
        const int r0 = blk * kDB, nrow = min(kDB, n - r0), r1 = r0 + nrow;
        PEEC_LAUNCH(k_trsm_diag<true>, dgrid, 256, 0, F, n, r0, nrow, Yt, nrhs, (const int *)done);
        if (r1 < n)
            PEEC_LAUNCH(k_cgemm_sub, dim3((nrhs + 63) / 64, (n - r1 + 63) / 64), 256, 0, F + (size_t)r1 * n + r0, n,
                        Yt + (size_t)r0 * nrhs, Yt + (size_t)r1 * nrhs, nrhs, n - r1, nrhs, nrow, (const int *)done);
    }
    for (int blk = nb - 1; blk >= 0; --blk) {  // backward: upper
        const int r0 = blk * kDB, nrow = min(kDB, n - r0);
        PEEC_LAUNCH(k_trsm_diag<false>, dgrid, 256, 0, F, n, r0, nrow, Yt, nrhs, (const int *)done);
        if (r0 > 0)
            PEEC_LAUNCH(k_cgemm_sub, dim3((nrhs + 63) / 64, (r0 + 63) / 64), 256, 0, F + r0, n,
                        Yt + (size_t)r0 * nrhs, Yt, nrhs, r0, nrhs, nrow, (const int *)done);
    }
    PEEC_LAUNCH(k_update_out, tgrid, 256, 0, (c64 *)x, Yt, cs, n, nrhs, (float4 *)xs, (const int *)done);
    PEEC_LAUNCH(k_residual_gemm_df, dim3((nrhs + 31) / 32, (n + 63) / 64), 256, sizeof(RTile), (const float4 *)Zs,
                (const float4 *)xs, (const c64 *)b, n, nrhs, (c64 *)r, be, be_q, (const int *)done);
    PEEC_LAUNCH(k_mark_done, qgrid, 256, 0, (const unsigned long long *)be_q, done, nrhs, tol);
    return launch_ok("many-right-hand-side sweep");
}

}  // namespace peec
