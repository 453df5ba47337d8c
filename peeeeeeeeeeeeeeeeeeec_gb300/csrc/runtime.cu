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

static std::once_flag g_pool_once;
static std::atomic<unsigned long long> g_launches{0};
static thread_local char g_err[512] = "";

// One non-blocking stream per host thread: calls from different threads (the
// serving loop's workers) overlap on the device; every entry point
// synchronises its own thread's stream before it returns host results.
struct ThreadStream {
    cudaStream_t s = nullptr;
    ~ThreadStream() {
        if (s) cudaStreamDestroy(s);
    }
};
static thread_local ThreadStream t_stream;

cudaStream_t stream() {
    std::call_once(g_pool_once, [] {
        // keep freed blocks in the stream-ordered pool between calls
        cudaMemPool_t pool;
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t threshold = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        }
    });
    if (!t_stream.s && cudaStreamCreateWithFlags(&t_stream.s, cudaStreamNonBlocking) != cudaSuccess)
        t_stream.s = nullptr;
    return t_stream.s;
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

// ---------------------------------------------------------------------
// FP64 / FP32 issue-rate probes: the roofline denominators for the FP64-
// and FP32-pipe kernels (the machine's measured peaks cover HBM and BF16 only).
// Independent FMA chains per thread, 8 CTAs per SM, CUDA-event timed.
// ---------------------------------------------------------------------
namespace peec {
__global__ void k_probe_dfma(double *out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
__global__ void k_probe_ffma(float *out, int iters, float a, float b) {
    float x[8];
    for (int j = 0; j < 8; ++j) x[j] = threadIdx.x * 1e-3f + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fmaf(x[j], a, b);
    }
    float s = 0;
    for (int j = 0; j < 8; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace peec

extern "C" int peec_gb300_pipe_peaks(double *fp64_tflops, double *fp32_tflops) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int blocks = sms * 8, threads = 256;
    size_t n = (size_t)blocks * threads;
    peec::DBuf<double> d(n);
    peec::DBuf<float> f(n);
    if (!d.p || !f.p) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float ms = 0;
    const int itd = 2048, itf = 32768;
    PEEC_LAUNCH(peec::k_probe_dfma, blocks, threads, 0, d.p, 16, 1.0000001, 1e-9);
    cudaEventRecord(e0, peec::stream());
    PEEC_LAUNCH(peec::k_probe_dfma, blocks, threads, 0, d.p, itd, 1.0000001, 1e-9);
    cudaEventRecord(e1, peec::stream());
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (fp64_tflops) *fp64_tflops = 2.0 * 4 * itd * (double)n / (ms * 1e9);
    PEEC_LAUNCH(peec::k_probe_ffma, blocks, threads, 0, f.p, 16, 1.0000001f, 1e-9f);
    cudaEventRecord(e0, peec::stream());
    PEEC_LAUNCH(peec::k_probe_ffma, blocks, threads, 0, f.p, itf, 1.0000001f, 1e-9f);
    cudaEventRecord(e1, peec::stream());
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (fp32_tflops) *fp32_tflops = 2.0 * 8 * itf * (double)n / (ms * 1e9);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return peec::sync("pipe peak probe") ? 0 : -1;
}
