// rts_peaks.cu -- measured ceilings that the roofline fractions of the FP64
// kernels and of the host-buffer calls divide by: the FP64 FMA throughput of
// the device (GB300 has no FP64 tensor path worth using, so the FP64 kernels
// run on the FP64 pipe of the SMs) and the host<->device copy rates of
// pinned memory.  No counterpart in the reference.
#include <chrono>
#include <cstring>

#include "rts_internal.h"

namespace {

constexpr int PEAK_CHAINS = 8;     // independent FMA chains per thread
constexpr int PEAK_THREADS = 256;  // per CTA
constexpr int PEAK_CTAS_PER_SM = 4;

// Every thread runs PEAK_CHAINS independent FMA chains x <- x * a + b for
// `iters` rounds (a < 1, so the values stay bounded); the sum is written only
// if it equals an impossible value, which keeps the chains live.
__global__ void __launch_bounds__(PEAK_THREADS) fp64_fma_kernel(double* sink, int64_t iters, double a, double b)
{
    double x[PEAK_CHAINS];
#pragma unroll
    for (int i = 0; i < PEAK_CHAINS; ++i) x[i] = 1e-3 * (threadIdx.x + i);
#pragma unroll 4
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < PEAK_CHAINS; ++i) x[i] = fma(x[i], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < PEAK_CHAINS; ++i) s += x[i];
    if (s == -1.0) sink[blockIdx.x] = s;
}

}  // namespace

extern "C" {

int rts_measure_fp64_peak(rts_ctx* ctx, double seconds, double* tflops)
{
    if (!ctx || !tflops) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, seconds > 0.0 && seconds <= 60.0, RTS_ERR_INVALID_ARGUMENT,
                "rts_measure_fp64_peak: %g s outside (0, 60]", seconds);
    RTS_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    const unsigned grid = (unsigned)(ctx->num_sms * PEAK_CTAS_PER_SM);
    void* sink = nullptr;
    int rc = rts_dmalloc(ctx, &sink, sizeof(double) * grid, "fp64 peak sink");
    if (rc != RTS_OK) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto done = [&](int r) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        rts_dfree(ctx, sink, sizeof(double) * grid);
        return r;
    };
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return done(rts_fail(ctx, RTS_ERR_CUDA, "rts_measure_fp64_peak: event creation failed"));
    // calibrate the round count on a short launch, then time one launch of
    // about `seconds`
    int64_t iters = 1 << 14;
    double best = 0.0;
    for (int pass = 0; pass < 3; ++pass) {
        cudaEventRecord(e0, st);
        fp64_fma_kernel<<<grid, PEAK_THREADS, 0, st>>>((double*)sink, iters, 0.999999, 1e-7);
        cudaEventRecord(e1, st);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e != cudaSuccess)
            return done(rts_fail(ctx, RTS_ERR_CUDA, "fp64_fma_kernel: %s", cudaGetErrorString(e)));
        ctx->launches++;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * PEAK_CHAINS * (double)iters * grid * PEAK_THREADS;
        if (pass > 0) best = flops / (ms * 1e-3) / 1e12 > best ? flops / (ms * 1e-3) / 1e12 : best;
        if (pass == 0) {
            const double per_iter = (ms * 1e-3) / (double)iters;
            iters = (int64_t)(seconds / 2 / (per_iter > 0 ? per_iter : 1e-9));
            if (iters < (1 << 14)) iters = 1 << 14;
        }
    }
    *tflops = best;
    return done(RTS_OK);
}

int rts_measure_link(rts_ctx* ctx, int64_t bytes, int reps, double* h2d_gbs, double* d2h_gbs, double* both_gbs)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, bytes >= (1 << 20) && reps >= 1 && reps <= 100, RTS_ERR_INVALID_ARGUMENT,
                "rts_measure_link: %lld bytes x %d repetitions", (long long)bytes, reps);
    RTS_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    void *dev_a = nullptr, *dev_b = nullptr, *host_a = nullptr, *host_b = nullptr;
    int rc = rts_dmalloc(ctx, &dev_a, (size_t)bytes, "link probe");
    if (rc == RTS_OK) rc = rts_dmalloc(ctx, &dev_b, (size_t)bytes, "link probe");
    cudaStream_t s_in = ctx->streams[RTS_STREAM_SCATTERING_1], s_out = ctx->streams[RTS_STREAM_SCATTERING_2];
    cudaEvent_t ev[7] = {};
    auto done = [&](int r) {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (host_a) cudaFreeHost(host_a);
        if (host_b) cudaFreeHost(host_b);
        rts_dfree(ctx, dev_a, (size_t)bytes);
        rts_dfree(ctx, dev_b, (size_t)bytes);
        return r;
    };
    if (rc != RTS_OK) return done(rc);
    if (cudaMallocHost(&host_a, (size_t)bytes) != cudaSuccess || cudaMallocHost(&host_b, (size_t)bytes) != cudaSuccess) {
        cudaGetLastError();
        return done(rts_fail(ctx, RTS_ERR_OUT_OF_MEMORY, "rts_measure_link: pinned host allocation failed"));
    }
    memset(host_a, 1, (size_t)bytes);
    memset(host_b, 2, (size_t)bytes);
    for (cudaEvent_t& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess)
            return done(rts_fail(ctx, RTS_ERR_CUDA, "rts_measure_link: event creation failed"));
    double best_in = 0.0, best_out = 0.0, best_both = 0.0;
    for (int r = 0; r <= reps; ++r) {  // the first round warms up
        float ms_in = 0.f, ms_out = 0.f, ms_both = 0.f;
        cudaEventRecord(ev[0], s_in);
        cudaMemcpyAsync(dev_a, host_a, (size_t)bytes, cudaMemcpyHostToDevice, s_in);
        cudaEventRecord(ev[1], s_in);
        cudaEventRecord(ev[2], s_in);
        cudaMemcpyAsync(host_b, dev_b, (size_t)bytes, cudaMemcpyDeviceToHost, s_in);
        cudaEventRecord(ev[3], s_in);
        // both directions at once: H2D on one stream, D2H on the other
        cudaEventRecord(ev[4], s_in);
        cudaStreamWaitEvent(s_out, ev[4], 0);
        cudaMemcpyAsync(dev_a, host_a, (size_t)bytes, cudaMemcpyHostToDevice, s_in);
        cudaMemcpyAsync(host_b, dev_b, (size_t)bytes, cudaMemcpyDeviceToHost, s_out);
        cudaEventRecord(ev[6], s_in);
        cudaStreamWaitEvent(s_out, ev[6], 0);  // the end event follows both copies
        cudaEventRecord(ev[5], s_out);
        cudaStreamWaitEvent(s_in, ev[5], 0);
        cudaError_t e = cudaStreamSynchronize(s_in);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s_out);
        if (e != cudaSuccess) return done(rts_fail(ctx, RTS_ERR_CUDA, "rts_measure_link: %s", cudaGetErrorString(e)));
        cudaEventElapsedTime(&ms_in, ev[0], ev[1]);
        cudaEventElapsedTime(&ms_out, ev[2], ev[3]);
        cudaEventElapsedTime(&ms_both, ev[4], ev[5]);
        if (r == 0) continue;
        const double gb = (double)bytes / 1e9;
        if (gb / (ms_in * 1e-3) > best_in) best_in = gb / (ms_in * 1e-3);
        if (gb / (ms_out * 1e-3) > best_out) best_out = gb / (ms_out * 1e-3);
        if (2 * gb / (ms_both * 1e-3) > best_both) best_both = 2 * gb / (ms_both * 1e-3);
    }
    if (h2d_gbs) *h2d_gbs = best_in;
    if (d2h_gbs) *d2h_gbs = best_out;
    if (both_gbs) *both_gbs = best_both;
    return done(RTS_OK);
}

}  // extern "C"
