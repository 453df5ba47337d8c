// Shared plumbing for the sm_103a PEEC library: error reporting, the
// library stream, stream-ordered device buffers and launch accounting.
//
// The whole library is compiled with --fmad=false: a*b+c is never contracted
// implicitly, so expressions that must match the reference's rounding (the
// patch classification, triangle maps, entry scaling) evaluate exactly as
// written.  Hot loops that want fused multiply-adds call fma() explicitly.
#pragma once

#include <cuda_runtime.h>
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

// Warp helpers.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}

}  // namespace peec

#define PEEC_LAUNCH(kernel, grid, block, smem, ...)                              \
    do {                                                                         \
        kernel<<<(grid), (block), (smem), ::peec::stream()>>>(__VA_ARGS__);      \
        ::peec::note_launch();                                                   \
    } while (0)
