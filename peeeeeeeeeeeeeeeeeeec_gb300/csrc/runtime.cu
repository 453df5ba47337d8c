// Library runtime: stream, errors, allocation, launch accounting and the
// small extension API (include/peec_gb300.h) for device-resident use.
#include "common.cuh"

#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "../../include/peec_gb300.h"

namespace peec {

static std::once_flag g_stream_once;
static cudaStream_t g_stream = nullptr;
static std::atomic<unsigned long long> g_launches{0};
static thread_local char g_err[512] = "";

cudaStream_t stream() {
    std::call_once(g_stream_once, [] {
        if (cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking) != cudaSuccess) g_stream = nullptr;
        // keep freed blocks in the pool between calls
        cudaMemPool_t pool;
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t threshold = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        }
    });
    return g_stream;
}

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    fprintf(stderr, "ERROR: %s\n", g_err);
}

const char *last_error() { return g_err; }

void note_launch(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(); }

bool cuda_ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    set_error("CUDA failure in %s: %s", what, cudaGetErrorString(e));
    return false;
}

bool launch_ok(const char *what) { return cuda_ok(cudaGetLastError(), what); }

void *dalloc(size_t bytes) {
    void *p = nullptr;
    if (bytes == 0) return nullptr;
    if (!cuda_ok(cudaMallocAsync(&p, bytes, stream()), "device allocation")) return nullptr;
    return p;
}

void dfree(void *p) {
    if (p) cudaFreeAsync(p, stream());
}

bool sync(const char *what) { return cuda_ok(cudaStreamSynchronize(stream()), what); }

}  // namespace peec

// ---------------------------------------------------------------------
// extension API
// ---------------------------------------------------------------------
extern "C" {

const char *peec_gb300_last_error(void) { return peec::last_error(); }

unsigned long long peec_gb300_launch_count(void) { return peec::launch_count(); }

int peec_gb300_device_ready(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return 0;
    return peec::stream() != nullptr;
}

void *peec_gb300_stream(void) { return (void *)peec::stream(); }

void *peec_gb300_device_alloc(size_t bytes) {
    void *p = nullptr;
    if (!peec::cuda_ok(cudaMalloc(&p, bytes ? bytes : 1), "device allocation")) return nullptr;
    return p;
}

void peec_gb300_device_free(void *p) {
    if (p) cudaFree(p);
}

int peec_gb300_copy_to_device(void *dst, const void *src, size_t bytes) {
    if (!peec::cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, peec::stream()), "copy"))
        return -1;
    return peec::sync("copy") ? 0 : -1;
}

int peec_gb300_copy_to_host(void *dst, const void *src, size_t bytes) {
    if (!peec::cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, peec::stream()), "copy"))
        return -1;
    return peec::sync("copy") ? 0 : -1;
}

int peec_gb300_copy_device(void *dst, const void *src, size_t bytes) {
    return peec::cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, peec::stream()), "copy") ? 0 : -1;
}

void *peec_gb300_host_alloc_pinned(size_t bytes) {
    void *p = nullptr;
    if (!peec::cuda_ok(cudaMallocHost(&p, bytes ? bytes : 1), "pinned allocation")) return nullptr;
    return p;
}

void peec_gb300_host_free_pinned(void *p) {
    if (p) cudaFreeHost(p);
}

int peec_gb300_synchronize(void) { return peec::sync("synchronize") ? 0 : -1; }

void *peec_gb300_event_record(void) {
    cudaEvent_t e;
    if (!peec::cuda_ok(cudaEventCreate(&e), "event")) return nullptr;
    if (!peec::cuda_ok(cudaEventRecord(e, peec::stream()), "event record")) {
        cudaEventDestroy(e);
        return nullptr;
    }
    return (void *)e;
}

double peec_gb300_event_elapsed_ms(void *start, void *stop) {
    float ms = -1.0f;
    if (!start || !stop) return -1.0;
    cudaEventSynchronize((cudaEvent_t)stop);
    if (cudaEventElapsedTime(&ms, (cudaEvent_t)start, (cudaEvent_t)stop) != cudaSuccess) return -1.0;
    return (double)ms;
}

void peec_gb300_event_destroy(void *e) {
    if (e) cudaEventDestroy((cudaEvent_t)e);
}

}  // extern "C"
