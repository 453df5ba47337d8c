// Shared plumbing for the sm_103a PEEC library: error reporting, the
// library stream, stream-ordered device buffers and launch accounting.
//
// The whole library is compiled with --fmad=false: a*b+c is never contracted
// implicitly, so expressions that must match the reference's rounding (the
// patch classification, triangle maps, entry scaling) evaluate exactly as
// written.  Hot loops that want fused multiply-adds call fma() explicitly.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stddef.h>

namespace peec {

// Library-wide stream (created on first use, non-blocking).  All entry
// points enqueue on it and synchronise it before returning host results.
cudaStream_t stream();

// Remember the last error text (thread-local), also printed with an
// "ERROR:" prefix to stderr as the reference's tests expect.
void set_error(const char *fmt, ...);
const char *last_error();

// Count of kernels launched by this library since load (for the bench's
// gpu_launches figure).  Every launch goes through note_launch().
void note_launch(int n = 1);
unsigned long long launch_count();

// Check a CUDA call; on failure record the error and return false.
bool cuda_ok(cudaError_t e, const char *what);

// After a launch: check the launch error.
bool launch_ok(const char *what);

// Stream-ordered device allocation on the library stream.
void *dalloc(size_t bytes);
void dfree(void *p);

template <class T> struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    explicit DBuf(size_t count) { alloc(count); }
    bool alloc(size_t count) {
        release();
        n = count;
        p = count ? static_cast<T *>(dalloc(count * sizeof(T))) : nullptr;
        return count == 0 || p != nullptr;
    }
    void release() {
        if (p) dfree(p);
        p = nullptr;
        n = 0;
    }
    ~DBuf() { release(); }
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    bool upload(const T *h, size_t count) {
        return cuda_ok(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, stream()),
                       "host->device copy");
    }
    bool download(T *h, size_t count) const {
        return cuda_ok(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, stream()),
                       "device->host copy");
    }
};

bool sync(const char *what);

// ---- correctly rounded hypot ----
// sqrt(x^2 + y^2) rounded to nearest, ties to even: the value the reference's
// C library returns for hypot (its hypot is correctly rounded; checked
// against exact rational arithmetic on 2e5 random and adversarial inputs).
// The LU's equilibration scales and pivot magnitudes use it, so that pivot
// candidates that tie to within an ulp (each row's largest entry divided by
// its own scale, on structured meshes) compare exactly as in the reference.
// Method: a first root from the scaled inputs, then an exact integer test of
// the candidate against the two rounding midpoints, s = a^2 + b^2 and the
// midpoint squares formed as 192-bit integers (s > m^2 moves the result up
// one ulp, s < m^2 at the lower midpoint moves it down; equality picks the
// even neighbour).  Results that would be subnormal take the library hypot.
struct U192 {
    unsigned long long w0, w1, w2;  // least significant limb first
};

// x * x << sh for x < 2^56, 0 <= sh < 64.
__device__ __forceinline__ U192 u192_sq_shl(unsigned long long x, int sh) {
    const unsigned long long lo = x * x, hi = __umul64hi(x, x);
    U192 r;
    if (sh == 0) {
        r.w0 = lo;
        r.w1 = hi;
        r.w2 = 0;
    } else {
        r.w0 = lo << sh;
        r.w1 = (hi << sh) | (lo >> (64 - sh));
        r.w2 = hi >> (64 - sh);
    }
    return r;
}

__device__ __forceinline__ U192 u192_add(U192 a, U192 b) {
    U192 r;
    r.w0 = a.w0 + b.w0;
    unsigned long long c = r.w0 < a.w0;
    r.w1 = a.w1 + b.w1 + c;
    c = (r.w1 < a.w1) || (c && r.w1 == a.w1);
    r.w2 = a.w2 + b.w2 + c;
    return r;
}

// -1, 0, +1 for a < b, a == b, a > b.
__device__ __forceinline__ int u192_cmp(U192 a, U192 b) {
    if (a.w2 != b.w2) return a.w2 < b.w2 ? -1 : 1;
    if (a.w1 != b.w1) return a.w1 < b.w1 ? -1 : 1;
    if (a.w0 != b.w0) return a.w0 < b.w0 ? -1 : 1;
    return 0;
}

__device__ __forceinline__ double hypot_cr(double x, double y) {
    double a = fabs(x), b = fabs(y);
    if (isinf(a) || isinf(b)) return INFINITY;
    if (isnan(a) || isnan(b)) return a + b;
    if (a < b) {
        const double t = a;
        a = b;
        b = t;
    }
    if (b == 0.0) return a;
    const int ea = ilogb(a), eb = ilogb(b);
    // b < a 2^-26: a^2 + b^2 < (a + ulp(a)/2)^2, so the result is a
    if (eb < ea - 27) return a;
    if (ea < -1000) return hypot(a, b);
    const int d = ea - eb;  // 0..27
    const unsigned long long A = (unsigned long long)scalbn(a, 52 - ea);
    const unsigned long long B = (unsigned long long)scalbn(b, 52 - eb);
    // 4 s 2^(104 - 2 ea + 2 d) as an integer
    const U192 S4 = u192_add(u192_sq_shl(A, 2 * d + 2), u192_sq_shl(B, 2));
    const U192 S16 = u192_add(u192_sq_shl(A, 2 * d + 4), u192_sq_shl(B, 4));
    const double a1 = scalbn(a, -ea), b1 = scalbn(b, -ea);
    double r = scalbn(sqrt(fma(a1, a1, b1 * b1)), ea);
    for (int it = 0; it < 3 && isfinite(r); ++it) {
        const int er = ilogb(r);
        const unsigned long long R = (unsigned long long)scalbn(r, 52 - er);
        const int sh = 2 * (er - ea) + 2 * d;
        // upper midpoint (2R + 1) 2^(er - 53)
        const int cu = u192_cmp(S4, u192_sq_shl(2 * R + 1, sh));
        if (cu > 0 || (cu == 0 && (R & 1))) {
            r = __longlong_as_double(__double_as_longlong(r) + 1);  // r > 0: next double up
            continue;
        }
        // lower midpoint: (2R - 1) 2^(er - 53), or (4R - 1) 2^(er - 54) when
        // r is a power of two (the lower neighbour's ulp is half of r's)
        const bool pow2 = R == (1ull << 52);
        const int cd = pow2 ? u192_cmp(S16, u192_sq_shl(4 * R - 1, sh)) : u192_cmp(S4, u192_sq_shl(2 * R - 1, sh));
        if (cd < 0 || (cd == 0 && (R & 1))) {
            r = __longlong_as_double(__double_as_longlong(r) - 1);  // next double down
            continue;
        }
        break;
    }
    return r;
}

// Warp helpers.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}

// Programmatic dependent launch: a kernel launched by pdl_launch may be
// scheduled while the previous kernel on the stream still runs; it calls
// pdl_wait() before touching any data, which returns once that kernel has
// completed and its memory is visible, and pdl_trigger() to let the next
// kernel be scheduled early in turn.  Both are no-ops in a kernel launched
// without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream();
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);  // an error stays the thread's last error (launch_ok)
    note_launch();
}

}  // namespace peec

#define PEEC_LAUNCH(kernel, grid, block, smem, ...)                              \
    do {                                                                         \
        kernel<<<(grid), (block), (smem), ::peec::stream()>>>(__VA_ARGS__);      \
        ::peec::note_launch();                                                   \
    } while (0)
