// rts_context.cu -- context, memory, transfers, synchronisation and the
// reference-compatible entry points of the C ABI (include/rts_scatter.h).
//
// Reference host layer this replaces (paths relative to solver_hllc_illum_cuda/):
//   SetDevice / CudaSyncStream / CudaWait ........ cuda/cuda_solve.cu:37-67
//   CudaSendIllumAsync / CopyIllumOnDevice ........ cuda/cuda_solve.cu:69-88
//   CalculateIntScattering* ........................ cuda/cuda_solve.cu:89-170
//   InitDevice / ClearDevice / ClearHost ........... cuda/cuda_struct.cu:134-214
// Differences by design: a context object instead of file-scope globals,
// status codes instead of exit(1), 64-bit sizes, an HBM budget, deadlines on
// every host-side wait.
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <thread>

#include "rts_internal.h"

int rts_fail(rts_ctx* ctx, int status, const char* fmt, ...)
{
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return status;
}

int rts_dmalloc(rts_ctx* ctx, void** p, size_t bytes, const char* what)
{
    *p = nullptr;
    if (bytes == 0) return RTS_OK;
    if (ctx->used_bytes + (int64_t)bytes > ctx->budget_bytes)
        return rts_fail(ctx, RTS_ERR_OVER_BUDGET,
                        "%s: %zu bytes would exceed the HBM budget (%lld of %lld bytes in use)",
                        what, bytes, (long long)ctx->used_bytes, (long long)ctx->budget_bytes);
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return rts_fail(ctx, RTS_ERR_OUT_OF_MEMORY, "%s: cudaMalloc(%zu) failed: %s", what, bytes,
                        cudaGetErrorString(e));
    }
    ctx->used_bytes += (int64_t)bytes;
    return RTS_OK;
}

void rts_dfree(rts_ctx* ctx, void* p, size_t bytes)
{
    if (!p) return;
    cudaFree(p);
    ctx->used_bytes -= (int64_t)bytes;
}

int rts_pmalloc(rts_ctx* ctx, void** p, size_t bytes, const char* what, cudaStream_t st)
{
    *p = nullptr;
    if (bytes == 0) return RTS_OK;
    if (ctx->used_bytes + (int64_t)bytes > ctx->budget_bytes)
        return rts_fail(ctx, RTS_ERR_OVER_BUDGET,
                        "%s: %zu bytes would exceed the HBM budget (%lld of %lld bytes in use)",
                        what, bytes, (long long)ctx->used_bytes, (long long)ctx->budget_bytes);
    if (!ctx->pool) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = ctx->device;
        RTS_CUDA_TRY(ctx, cudaMemPoolCreate(&ctx->pool, &props));
        uint64_t keep = UINT64_MAX;  // keep freed memory in the pool for the next problem
        RTS_CUDA_TRY(ctx, cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, ctx->pool, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return rts_fail(ctx, RTS_ERR_OUT_OF_MEMORY, "%s: pool allocation of %zu bytes failed: %s", what, bytes,
                        cudaGetErrorString(e));
    }
    ctx->used_bytes += (int64_t)bytes;
    return RTS_OK;
}

void rts_pfree(rts_ctx* ctx, void* p, size_t bytes, cudaStream_t st)
{
    if (!p) return;
    cudaFreeAsync(p, st);
    ctx->used_bytes -= (int64_t)bytes;
}

static void free_grid(rts_ctx* ctx)
{
    const int64_t loc = ctx->local();
    rts_split_free(ctx);
    rts_sweep_free(ctx);
    rts_dfree(ctx, ctx->d_illum, rts_bytes<double>(ctx->M * ctx->N * 4));
    rts_dfree(ctx, ctx->d_S, rts_bytes<double>(loc * ctx->N));
    rts_dfree(ctx, ctx->d_W, rts_bytes<double>(ctx->M * loc));
    rts_dfree(ctx, ctx->d_energy, rts_bytes<double>(ctx->N));
    rts_dfree(ctx, ctx->d_flux, rts_bytes<double>(ctx->N * 3));
    rts_dfree(ctx, ctx->d_geo, rts_bytes<double>(ctx->N * 17));
    rts_dfree(ctx, ctx->d_params, rts_bytes<double>(ctx->N * 17));
    ctx->d_geo = ctx->d_params = nullptr;
    rts_dfree(ctx, ctx->d_B, rts_bytes<double>(ctx->N));
    rts_dfree(ctx, ctx->d_xyz, rts_bytes<double>(ctx->M * 3));
    rts_dfree(ctx, ctx->d_area, rts_bytes<double>(ctx->M));
    if (ctx->h_illum) cudaFreeHost(ctx->h_illum);
    if (ctx->h_S) cudaFreeHost(ctx->h_S);
    ctx->d_illum = ctx->d_S = ctx->d_W = ctx->d_energy = ctx->d_flux = ctx->d_B = nullptr;
    ctx->d_xyz = ctx->d_area = nullptr;
    ctx->h_illum = ctx->h_S = nullptr;
    ctx->N = ctx->M = 0;
    ctx->out_start = ctx->out_end = 0;
    rts_inputs_changed(ctx);
    ctx->solve_has_prev = false;
}

static bool valid_stream(int s) { return s >= 0 && s < RTS_STREAM_COUNT; }

// Orders an integral call on `stream` after the writes of its device inputs
// (the Illum copies and every other rewrite of the Illum, W or scattering
// array queued on the scattering stream), but not after the integral calls
// queued there since: the mark is recorded on the scattering stream at the
// first integral call after such a write, before that call's own work.  The
// reference's pair of calls on scattering streams 1 and 2
// (solve_module/illum/Illum_async.cpp:1019-1020) then overlaps, one call's
// D2H with the other's integral, as the reference's unordered streams do.
static int after_input_writes(rts_ctx* ctx, int stream)
{
    cudaStream_t s1 = ctx->streams[RTS_STREAM_SCATTERING_1];
    if (!ctx->ev_inputs) RTS_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->ev_inputs, cudaEventDisableTiming));
    if (!ctx->inputs_marked) {
        RTS_CUDA_TRY(ctx, cudaEventRecord(ctx->ev_inputs, s1));
        ctx->inputs_marked = true;
    }
    if (stream != RTS_STREAM_SCATTERING_1) RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->streams[stream], ctx->ev_inputs, 0));
    return RTS_OK;
}

// Orders stream slot `stream` after the work already queued on the
// scattering stream (where the Illum copies go), with the context's event of
// that slot: recording and waiting capture the event's state at the call, so
// one event per waiting stream is enough.
static int after_scattering_stream(rts_ctx* ctx, int stream)
{
    if (stream == RTS_STREAM_SCATTERING_1) return RTS_OK;
    cudaEvent_t& ev = ctx->ev_order[stream];
    if (!ev) RTS_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    RTS_CUDA_TRY(ctx, cudaEventRecord(ev, ctx->streams[RTS_STREAM_SCATTERING_1]));
    RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->streams[stream], ev, 0));
    return RTS_OK;
}

void rts_timing_begin(rts_ctx* ctx, cudaStream_t st)
{
    if (!ctx->timing) return;
    if (ctx->tev_used + 2 > ctx->tev.size()) {
        for (int i = 0; i < 64; ++i) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) {
                cudaGetLastError();
                ctx->timing = false;
                return;
            }
            ctx->tev.push_back(e);
        }
    }
    cudaEventRecord(ctx->tev[ctx->tev_used], st);
}

void rts_timing_end(rts_ctx* ctx, cudaStream_t st)
{
    if (!ctx->timing || ctx->tev_used + 2 > ctx->tev.size()) return;
    cudaEventRecord(ctx->tev[ctx->tev_used + 1], st);
    ctx->tev_used += 2;
}

extern "C" {

int rts_abi_version(void) { return RTS_ABI_VERSION; }

int rts_ctx_create(int device, rts_ctx** out)
{
    if (!out) return RTS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return RTS_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return RTS_ERR_INVALID_ARGUMENT;
    rts_ctx* ctx = new rts_ctx();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete ctx;
        return RTS_ERR_CUDA;
    }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    ctx->num_sms = prop.multiProcessorCount;
    ctx->cc_major = prop.major;
    ctx->cc_minor = prop.minor;
    // Priorities as SetDevice: params high, scattering_1 middle, scattering_2 low.
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    const int prio[RTS_STREAM_COUNT] = {(prio_high + prio_low) / 2, prio_low, prio_high};
    for (int i = 0; i < RTS_STREAM_COUNT; ++i) {
        if (cudaStreamCreateWithPriority(&ctx->streams[i], cudaStreamNonBlocking, prio[i]) !=
            cudaSuccess) {
            rts_ctx_destroy(ctx);
            return RTS_ERR_CUDA;
        }
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    ctx->budget_bytes = (int64_t)(0.9 * (double)free_b);
    void* p = nullptr;
    if (rts_dmalloc(ctx, &p, sizeof(unsigned long long) * (RTS_RESID_CAP + 1), "residual") != RTS_OK) {
        rts_ctx_destroy(ctx);
        return RTS_ERR_OUT_OF_MEMORY;
    }
    ctx->d_resid = (unsigned long long*)p;
    ctx->resid_target = ctx->d_resid;
    if (rts_dmalloc(ctx, &p, sizeof(int) * 4, "flags") != RTS_OK) {
        rts_ctx_destroy(ctx);
        return RTS_ERR_OUT_OF_MEMORY;
    }
    ctx->d_flag = (int*)p;
    cudaMemset(ctx->d_resid, 0, sizeof(unsigned long long) * (RTS_RESID_CAP + 1));
    cudaMemset(ctx->d_flag, 0, sizeof(int) * 4);
    *out = ctx;
    return RTS_OK;
}

int rts_ctx_destroy(rts_ctx* ctx)
{
    if (!ctx) return RTS_OK;
    cudaSetDevice(ctx->device);
    for (int i = 0; i < RTS_STREAM_COUNT; ++i)
        if (ctx->streams[i]) cudaStreamSynchronize(ctx->streams[i]);
    free_grid(ctx);
    rts_dfree(ctx, ctx->d_resid, sizeof(unsigned long long) * (RTS_RESID_CAP + 1));
    rts_dfree(ctx, ctx->d_flag, sizeof(int) * 4);
    for (int i = 0; i < RTS_STREAM_COUNT; ++i)
        if (ctx->streams[i]) cudaStreamSynchronize(ctx->streams[i]);
    if (ctx->serve_copy) {
        cudaStreamSynchronize(ctx->serve_copy);
        cudaStreamDestroy(ctx->serve_copy);
    }
    if (ctx->serve_admit) {
        cudaStreamSynchronize(ctx->serve_admit);
        cudaStreamDestroy(ctx->serve_admit);
    }
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    for (int i = 0; i < RTS_STREAM_COUNT; ++i)
        if (ctx->streams[i]) cudaStreamDestroy(ctx->streams[i]);
    for (cudaEvent_t e : ctx->tev) cudaEventDestroy(e);
    for (int i = 0; i < RTS_STREAM_COUNT; ++i) {
        if (ctx->ev_order[i]) cudaEventDestroy(ctx->ev_order[i]);
        if (ctx->ev_sync[i]) cudaEventDestroy(ctx->ev_sync[i]);
    }
    if (ctx->ev_inputs) cudaEventDestroy(ctx->ev_inputs);
    delete ctx;
    return RTS_OK;
}

const char* rts_last_error(const rts_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int rts_set_hbm_budget(rts_ctx* ctx, int64_t bytes)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, bytes >= ctx->used_bytes, RTS_ERR_OVER_BUDGET,
                "budget %lld below the %lld bytes already held", (long long)bytes,
                (long long)ctx->used_bytes);
    ctx->budget_bytes = bytes;
    return RTS_OK;
}

int rts_hbm_used(const rts_ctx* ctx, int64_t* bytes)
{
    if (!ctx || !bytes) return RTS_ERR_INVALID_ARGUMENT;
    *bytes = ctx->used_bytes;
    return RTS_OK;
}

int rts_init(rts_ctx* ctx, const double* xyz, const double* area, int64_t M, double full_area,
             int64_t N, int64_t start, int64_t end)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, xyz && area, RTS_ERR_INVALID_ARGUMENT, "rts_init: null direction arrays");
    RTS_REQUIRE(ctx, M > 0 && N > 0, RTS_ERR_INVALID_ARGUMENT,
                "rts_init: M=%lld and N=%lld must be positive", (long long)M, (long long)N);
    RTS_REQUIRE(ctx, 0 <= start && start < end && end <= M, RTS_ERR_INVALID_ARGUMENT,
                "rts_init: out-direction range [%lld,%lld) outside [0,%lld)", (long long)start,
                (long long)end, (long long)M);
    RTS_REQUIRE(ctx, full_area > 0.0, RTS_ERR_INVALID_ARGUMENT, "rts_init: full_area <= 0");
    RTS_REQUIRE(ctx, M <= (int64_t)1 << 20 && N <= (int64_t)1 << 40, RTS_ERR_INVALID_ARGUMENT,
                "rts_init: sizes out of range");
    RTS_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    for (int i = 0; i < RTS_STREAM_COUNT; ++i) cudaStreamSynchronize(ctx->streams[i]);
    free_grid(ctx);

    ctx->M = M;
    ctx->N = N;
    ctx->out_start = start;
    ctx->out_end = end;
    ctx->full_area = full_area;
    ctx->h_xyz.assign(xyz, xyz + 3 * M);
    ctx->h_area.assign(area, area + M);
    ctx->phase = RTS_PHASE_THOMSON;
    ctx->phase_g = 0.0;
    const int64_t loc = end - start;

    int st;
    void* p;
#define RTS_ALLOC(field, type, count, name)                                                 \
    if ((st = rts_dmalloc(ctx, &p, rts_bytes<type>(count), name)) != RTS_OK) {            \
        ctx->N = N;                                                                        \
        free_grid(ctx);                                                                    \
        return st;                                                                         \
    }                                                                                      \
    ctx->field = (type*)p;
    RTS_ALLOC(d_xyz, double, M * 3, "directions");
    RTS_ALLOC(d_area, double, M, "direction areas");
    RTS_ALLOC(d_illum, double, M * N * 4, "Illum");
    RTS_ALLOC(d_S, double, loc * N, "scattering");
    RTS_ALLOC(d_W, double, M * loc, "direction-pair weights");
    RTS_ALLOC(d_energy, double, N, "energy");
    RTS_ALLOC(d_flux, double, N * 3, "flux");
    RTS_ALLOC(d_B, double, N, "source B");
#undef RTS_ALLOC
    if (cudaMallocHost((void**)&ctx->h_illum, rts_bytes<double>(M * N * 4)) != cudaSuccess ||
        cudaMallocHost((void**)&ctx->h_S, rts_bytes<double>(loc * N)) != cudaSuccess) {
        cudaGetLastError();
        free_grid(ctx);
        return rts_fail(ctx, RTS_ERR_OUT_OF_MEMORY, "rts_init: pinned host allocation failed");
    }
    RTS_CUDA_TRY(ctx, cudaMemcpy(ctx->d_xyz, xyz, rts_bytes<double>(M * 3), cudaMemcpyHostToDevice));
    RTS_CUDA_TRY(ctx, cudaMemcpy(ctx->d_area, area, rts_bytes<double>(M), cudaMemcpyHostToDevice));
    RTS_CUDA_TRY(ctx, cudaMemset(ctx->d_S, 0, rts_bytes<double>(loc * N)));
    ctx->w_version++;
    return rts_launch_weights(ctx);
}

int rts_host_illum(rts_ctx* ctx, double** illum)
{
    if (!ctx || !illum) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->h_illum, RTS_ERR_BAD_STATE, "rts_host_illum before rts_init");
    *illum = ctx->h_illum;
    return RTS_OK;
}

int rts_host_scattering(rts_ctx* ctx, double** scattering)
{
    if (!ctx || !scattering) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->h_S, RTS_ERR_BAD_STATE, "rts_host_scattering before rts_init");
    *scattering = ctx->h_S;
    return RTS_OK;
}

int rts_set_phase(rts_ctx* ctx, int phase, double g)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_W, RTS_ERR_BAD_STATE, "rts_set_phase before rts_init");
    RTS_REQUIRE(ctx, phase == RTS_PHASE_THOMSON || phase == RTS_PHASE_HG, RTS_ERR_INVALID_ARGUMENT,
                "rts_set_phase: unknown phase %d", phase);
    RTS_REQUIRE(ctx, phase != RTS_PHASE_HG || (g > -1.0 && g < 1.0), RTS_ERR_INVALID_ARGUMENT,
                "rts_set_phase: HG asymmetry g=%g outside (-1,1)", g);
    ctx->phase = phase;
    ctx->phase_g = g;
    rts_inputs_changed(ctx);
    ctx->w_version++;
    return rts_launch_weights(ctx);
}

int rts_set_weights(rts_ctx* ctx, const double* W)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_W, RTS_ERR_BAD_STATE, "rts_set_weights before rts_init");
    RTS_REQUIRE(ctx, W, RTS_ERR_INVALID_ARGUMENT, "rts_set_weights: null W");
    RTS_CUDA_TRY(ctx, cudaMemcpy(ctx->d_W, W, rts_bytes<double>(ctx->M * ctx->local()),
                                 cudaMemcpyHostToDevice));
    ctx->phase = RTS_PHASE_CUSTOM;
    rts_inputs_changed(ctx);
    ctx->w_version++;
    return RTS_OK;
}

int rts_send_illum_async(rts_ctx* ctx, int64_t size, int64_t shift_dev, int64_t shift_host,
                         const double* illum_host)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_send_illum_async before rts_init");
    RTS_REQUIRE(ctx, illum_host, RTS_ERR_INVALID_ARGUMENT, "rts_send_illum_async: null host pointer");
    const int64_t total = ctx->M * ctx->N * 4;
    RTS_REQUIRE(ctx, size >= 0 && shift_dev >= 0 && shift_host >= 0 && shift_dev + size <= total,
                RTS_ERR_INVALID_ARGUMENT,
                "rts_send_illum_async: [%lld, %lld) outside the device Illum of %lld doubles",
                (long long)shift_dev, (long long)(shift_dev + size), (long long)total);
    if (size == 0) return RTS_OK;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_illum + shift_dev, illum_host + shift_host,
                                      rts_bytes<double>(size), cudaMemcpyHostToDevice,
                                      ctx->streams[RTS_STREAM_SCATTERING_1]));
    rts_inputs_changed(ctx);
    // at a tensor precision the integral calls' face sums start as the
    // directions arrive
    if (ctx->call_precision != RTS_PREC_FP64) return rts_split_eager_send(ctx, shift_dev, size);
    return RTS_OK;
}

int rts_copy_illum(rts_ctx* ctx, int64_t size, const double* illum_host)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_copy_illum before rts_init");
    RTS_REQUIRE(ctx, illum_host, RTS_ERR_INVALID_ARGUMENT, "rts_copy_illum: null host pointer");
    RTS_REQUIRE(ctx, size >= 0 && size <= ctx->M * ctx->N * 4, RTS_ERR_INVALID_ARGUMENT,
                "rts_copy_illum: size %lld exceeds the device Illum", (long long)size);
    RTS_CUDA_TRY(ctx, cudaMemcpy(ctx->d_illum, illum_host, rts_bytes<double>(size),
                                 cudaMemcpyHostToDevice));
    rts_inputs_changed(ctx);
    return RTS_OK;
}

int rts_read_illum(rts_ctx* ctx, int64_t size, double* illum_host)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_read_illum before rts_init");
    RTS_REQUIRE(ctx, illum_host, RTS_ERR_INVALID_ARGUMENT, "rts_read_illum: null host pointer");
    RTS_REQUIRE(ctx, size >= 0 && size <= ctx->M * ctx->N * 4, RTS_ERR_INVALID_ARGUMENT,
                "rts_read_illum: size %lld exceeds the device Illum", (long long)size);
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(illum_host, ctx->d_illum, rts_bytes<double>(size),
                                      cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

int rts_scattering_async(rts_ctx* ctx, int64_t start, int64_t end, int stream, double* host_out)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_S, RTS_ERR_BAD_STATE, "rts_scattering_async before rts_init");
    RTS_REQUIRE(ctx, valid_stream(stream), RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    RTS_REQUIRE(ctx, 0 <= start && start <= end && end <= ctx->local(), RTS_ERR_INVALID_ARGUMENT,
                "rts_scattering_async: [%lld,%lld) outside the %lld local out-directions",
                (long long)start, (long long)end, (long long)ctx->local());
    if (start == end) return RTS_OK;
    cudaStream_t st = ctx->streams[stream];
    int rc = after_input_writes(ctx, stream);
    if (rc != RTS_OK) return rc;
    if (ctx->call_precision == RTS_PREC_FP64)
        rc = rts_launch_scatter_fp64(ctx, start, end, st, nullptr, 0.0, false, false);
    else
        rc = rts_split_async(ctx, ctx->call_precision, start, end, stream, st);
    if (rc != RTS_OK) return rc;
    double* dst = host_out ? host_out : ctx->h_S;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(dst + start * ctx->N, ctx->d_S + start * ctx->N,
                                      rts_bytes<double>((end - start) * ctx->N),
                                      cudaMemcpyDeviceToHost, st));
    return RTS_OK;
}

int rts_scattering(rts_ctx* ctx, const double* illum_host, double* host_out)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_S, RTS_ERR_BAD_STATE, "rts_scattering before rts_init");
    const double* src = illum_host ? illum_host : ctx->h_illum;
    double* dst = host_out ? host_out : ctx->h_S;
    if (ctx->call_precision != RTS_PREC_FP64) {  // the bare integral at that precision, pipelined over cell ranges
        rts_inputs_changed(ctx);
        return rts_split_host_call(ctx, ctx->call_precision, src, nullptr, 1.0, dst);
    }
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_illum, src, rts_bytes<double>(ctx->M * ctx->N * 4),
                                      cudaMemcpyHostToDevice, st));
    rts_inputs_changed(ctx);
    int rc = rts_launch_scatter_fp64(ctx, 0, ctx->local(), st, nullptr, 0.0, false, false);
    if (rc != RTS_OK) return rc;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(dst, ctx->d_S, rts_bytes<double>(ctx->local() * ctx->N),
                                      cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

int rts_scattering_update(rts_ctx* ctx, int precision, const double* illum_host,
                          const double* B_host, double lambda, double* S_host)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_S, RTS_ERR_BAD_STATE, "rts_scattering_update before rts_init");
    RTS_REQUIRE(ctx, illum_host && S_host, RTS_ERR_INVALID_ARGUMENT,
                "rts_scattering_update: null host buffer");
    RTS_REQUIRE(ctx, B_host || lambda == 1.0, RTS_ERR_INVALID_ARGUMENT,
                "rts_scattering_update: B is required unless lambda == 1");
    if (precision == RTS_PREC_BF16X3 || precision == RTS_PREC_FP16X3 || precision == RTS_PREC_TF32X3) {
        rts_inputs_changed(ctx);
        return rts_split_host_call(ctx, precision, illum_host, B_host, lambda, S_host);
    }
    RTS_REQUIRE(ctx, precision == RTS_PREC_FP64, RTS_ERR_INVALID_ARGUMENT, "unknown precision %d", precision);
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_illum, illum_host,
                                      rts_bytes<double>(ctx->M * ctx->N * 4),
                                      cudaMemcpyHostToDevice, st));
    rts_inputs_changed(ctx);
    const bool update = B_host != nullptr && lambda != 1.0;
    if (update)
        RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_B, B_host, rts_bytes<double>(ctx->N),
                                          cudaMemcpyHostToDevice, st));
    int rc = rts_launch_scatter_fp64(ctx, 0, ctx->local(), st, ctx->d_B, lambda, update, false);
    if (rc != RTS_OK) return rc;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(S_host, ctx->d_S, rts_bytes<double>(ctx->local() * ctx->N),
                                      cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

int rts_read_scattering(rts_ctx* ctx, int64_t start, int64_t end, int stream, double* host_out)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_S, RTS_ERR_BAD_STATE, "rts_read_scattering before rts_init");
    RTS_REQUIRE(ctx, valid_stream(stream), RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    RTS_REQUIRE(ctx, 0 <= start && start <= end && end <= ctx->local(), RTS_ERR_INVALID_ARGUMENT,
                "rts_read_scattering: bad row range");
    if (start == end) return RTS_OK;
    double* dst = host_out ? host_out : ctx->h_S;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(dst + start * ctx->N, ctx->d_S + start * ctx->N,
                                      rts_bytes<double>((end - start) * ctx->N),
                                      cudaMemcpyDeviceToHost, ctx->streams[stream]));
    return RTS_OK;
}

int rts_send_scattering(rts_ctx* ctx, int64_t start, int64_t end, int stream, const double* host)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_S, RTS_ERR_BAD_STATE, "rts_send_scattering before rts_init");
    RTS_REQUIRE(ctx, valid_stream(stream), RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    RTS_REQUIRE(ctx, host, RTS_ERR_INVALID_ARGUMENT, "rts_send_scattering: null host array");
    RTS_REQUIRE(ctx, 0 <= start && start <= end && end <= ctx->local(), RTS_ERR_INVALID_ARGUMENT,
                "rts_send_scattering: [%lld,%lld) outside the %lld local out-directions", (long long)start,
                (long long)end, (long long)ctx->local());
    if (start == end) return RTS_OK;
    rts_inputs_changed(ctx);
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_S + start * ctx->N, host + start * ctx->N,
                                      rts_bytes<double>((end - start) * ctx->N), cudaMemcpyHostToDevice,
                                      ctx->streams[stream]));
    return RTS_OK;
}

int rts_device_arrays(rts_ctx* ctx, double** d_illum, double** d_scattering)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_S, RTS_ERR_BAD_STATE, "rts_device_arrays before rts_init");
    if (d_illum) *d_illum = ctx->d_illum;
    if (d_scattering) *d_scattering = ctx->d_S;
    return RTS_OK;
}

int rts_moments(rts_ctx* ctx, int stream, double* energy, double* flux)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_moments before rts_init");
    RTS_REQUIRE(ctx, valid_stream(stream), RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    cudaStream_t st = ctx->streams[stream];
    int rc = after_scattering_stream(ctx, stream);
    if (rc != RTS_OK) return rc;
    rc = rts_launch_moments(ctx, st);
    if (rc != RTS_OK) return rc;
    if (energy)
        RTS_CUDA_TRY(ctx, cudaMemcpyAsync(energy, ctx->d_energy, rts_bytes<double>(ctx->N),
                                          cudaMemcpyDeviceToHost, st));
    if (flux)
        RTS_CUDA_TRY(ctx, cudaMemcpyAsync(flux, ctx->d_flux, rts_bytes<double>(ctx->N * 3),
                                          cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

int rts_set_geometry(rts_ctx* ctx, const double* normals, const double* face_areas, const double* volume)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_set_geometry before rts_init");
    RTS_REQUIRE(ctx, normals && face_areas && volume, RTS_ERR_INVALID_ARGUMENT, "rts_set_geometry: null array");
    const int64_t N = ctx->N;
    for (int64_t c = 0; c < N; ++c)
        RTS_REQUIRE(ctx, volume[c] > 0.0, RTS_ERR_INVALID_ARGUMENT, "rts_set_geometry: volume[%lld] <= 0",
                    (long long)c);
    if (!ctx->d_geo) {
        void* p = nullptr;
        int rc = rts_dmalloc(ctx, &p, rts_bytes<double>(N * 17), "cell geometry");
        if (rc != RTS_OK) return rc;
        ctx->d_geo = (double*)p;
    }
    cudaStream_t st = ctx->streams[RTS_STREAM_PARAMS];
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_geo, normals, rts_bytes<double>(N * 12), cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_geo + 12 * N, face_areas, rts_bytes<double>(N * 4),
                                      cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_geo + 16 * N, volume, rts_bytes<double>(N), cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

int rts_illum_params(rts_ctx* ctx, int stream, double* energy, double* flux, double* impuls, double* divstream,
                     double* divimpuls)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_illum_params before rts_init");
    RTS_REQUIRE(ctx, valid_stream(stream), RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    RTS_REQUIRE(ctx, ctx->d_geo || (!divstream && !divimpuls), RTS_ERR_BAD_STATE,
                "the divergences need the cell geometry (rts_set_geometry)");
    const int64_t N = ctx->N;
    if (!ctx->d_params) {
        void* p = nullptr;
        int rc = rts_dmalloc(ctx, &p, rts_bytes<double>(N * 17), "illumination parameters");
        if (rc != RTS_OK) return rc;
        ctx->d_params = (double*)p;
    }
    cudaStream_t st = ctx->streams[stream];
    int rc = after_scattering_stream(ctx, stream);  // after the Illum copies queued on the scattering stream
    if (rc != RTS_OK) return rc;
    rc = rts_launch_illum_params(ctx, st);
    if (rc != RTS_OK) return rc;
    double* const d = ctx->d_params;
    struct {
        double* host;
        const double* dev;
        int64_t n;
    } outs[5] = {{energy, d, N}, {flux, d + N, 3 * N}, {impuls, d + 4 * N, 9 * N}, {divstream, d + 13 * N, N},
                 {divimpuls, d + 14 * N, 3 * N}};
    for (auto& o : outs)
        if (o.host)
            RTS_CUDA_TRY(ctx, cudaMemcpyAsync(o.host, o.dev, rts_bytes<double>(o.n), cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

int rts_source_update(rts_ctx* ctx, const double* B_host, double lambda, int64_t start,
                      int64_t end, int stream, double* residual)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_S, RTS_ERR_BAD_STATE, "rts_source_update before rts_init");
    RTS_REQUIRE(ctx, B_host, RTS_ERR_INVALID_ARGUMENT, "rts_source_update: null B");
    RTS_REQUIRE(ctx, valid_stream(stream), RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    RTS_REQUIRE(ctx, 0 <= start && start <= end && end <= ctx->local(), RTS_ERR_INVALID_ARGUMENT,
                "rts_source_update: bad row range");
    cudaStream_t st = ctx->streams[stream];
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_B, B_host, rts_bytes<double>(ctx->N),
                                      cudaMemcpyHostToDevice, st));
    ctx->resid_target = ctx->d_resid;
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_resid, 0, sizeof(unsigned long long), st));
    int rc = rts_launch_update(ctx, start, end, st, ctx->d_B, lambda, residual != nullptr);
    if (rc != RTS_OK) return rc;
    if (residual) {
        unsigned long long bits = 0;
        RTS_CUDA_TRY(ctx, cudaMemcpyAsync(&bits, ctx->d_resid, sizeof(bits),
                                          cudaMemcpyDeviceToHost, st));
        RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        memcpy(residual, &bits, sizeof(double));
    } else {
        RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    }
    return RTS_OK;
}

static int wait_event_deadline(rts_ctx* ctx, cudaEvent_t ev, int64_t timeout_us)
{
    if (timeout_us < 0) {
        RTS_CUDA_TRY(ctx, cudaEventSynchronize(ev));
        return RTS_OK;
    }
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t q = cudaEventQuery(ev);
        if (q == cudaSuccess) return RTS_OK;
        if (q != cudaErrorNotReady)
            return rts_fail(ctx, RTS_ERR_CUDA, "stream wait failed: %s", cudaGetErrorString(q));
        auto el = std::chrono::duration_cast<std::chrono::microseconds>(
                      std::chrono::steady_clock::now() - t0)
                      .count();
        if (el >= timeout_us)
            return rts_fail(ctx, RTS_ERR_TIMEOUT, "stream work not finished after %lld us",
                            (long long)timeout_us);
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

int rts_sync_stream(rts_ctx* ctx, int stream, int64_t timeout_us)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, valid_stream(stream), RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    cudaEvent_t& ev = ctx->ev_sync[stream];
    if (!ev) RTS_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    RTS_CUDA_TRY(ctx, cudaEventRecord(ev, ctx->streams[stream]));
    return wait_event_deadline(ctx, ev, timeout_us);
}

int rts_wait(rts_ctx* ctx, int64_t timeout_us)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < RTS_STREAM_COUNT; ++i) {
        int rc = rts_sync_stream(ctx, i, timeout_us);
        if (rc != RTS_OK) return rc;
    }
    return RTS_OK;
}

// ---------------------------------------------------------------------------
// device-resident source iteration
// ---------------------------------------------------------------------------

int rts_solve_setup(rts_ctx* ctx, int precision, const double* B_host, double lambda)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_S, RTS_ERR_BAD_STATE, "rts_solve_setup before rts_init");
    RTS_REQUIRE(ctx, B_host, RTS_ERR_INVALID_ARGUMENT, "rts_solve_setup: null B");
    RTS_REQUIRE(ctx, ctx->out_start == 0 && ctx->out_end == ctx->M, RTS_ERR_UNSUPPORTED,
                "rts_solve_setup needs all M out-directions local (got [%lld,%lld) of %lld)",
                (long long)ctx->out_start, (long long)ctx->out_end, (long long)ctx->M);
    RTS_REQUIRE(ctx,
                precision == RTS_PREC_FP64 || precision == RTS_PREC_BF16X3 ||
                    precision == RTS_PREC_FP16X3 || precision == RTS_PREC_TF32X3,
                RTS_ERR_INVALID_ARGUMENT, "rts_solve_setup: unknown precision %d", precision);
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_B, B_host, rts_bytes<double>(ctx->N),
                                      cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_S, 0, rts_bytes<double>(ctx->M * ctx->N), st));
    rts_inputs_written(ctx);  // S cleared; the steps relax the Illum
    ctx->solve_precision = precision;
    ctx->solve_lambda = lambda;
    ctx->solve_has_prev = false;
    ctx->solve_steps = 0;
    if (precision != RTS_PREC_FP64) {
        int rc = rts_split_setup(ctx, precision);
        if (rc != RTS_OK) return rc;
    }
    ctx->solve_ready = true;
    return RTS_OK;
}

int rts_solve_step_async(rts_ctx* ctx, int relax)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->solve_ready, RTS_ERR_BAD_STATE,
                "rts_solve_step before rts_solve_setup (or the inputs changed since)");
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    ctx->resid_target = ctx->d_resid + 1 + (ctx->solve_steps % RTS_RESID_CAP);
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(ctx->resid_target, 0, sizeof(unsigned long long), st));
    int rc;
    if (ctx->solve_precision == RTS_PREC_FP64) {
        rc = rts_launch_scatter_fp64(ctx, 0, ctx->M, st, ctx->d_B, ctx->solve_lambda, true, true);
        if (rc == RTS_OK && relax) rc = rts_launch_relax_fp64(ctx, st);
    } else {
        rc = rts_split_step(ctx, relax != 0, st);
    }
    rts_inputs_written(ctx);
    ctx->solve_has_prev = true;
    ctx->solve_steps++;
    return rc;
}

static int check_device_flag(rts_ctx* ctx)
{
    int flag = 0;
    RTS_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag)
        return rts_fail(ctx, RTS_ERR_DEVICE_WAIT,
                        "a bounded device-side wait gave up (code %d); results are invalid", flag);
    return RTS_OK;
}

int rts_solve_residual_history(rts_ctx* ctx, double* out, int64_t n)
{
    if (!ctx || (n > 0 && !out) || n < 0) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, n <= ctx->solve_steps && n <= RTS_RESID_CAP, RTS_ERR_INVALID_ARGUMENT,
                "rts_solve_residual_history: %lld steps requested, %lld kept", (long long)n,
                (long long)(ctx->solve_steps < RTS_RESID_CAP ? ctx->solve_steps : RTS_RESID_CAP));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->streams[RTS_STREAM_SCATTERING_1]));
    std::vector<unsigned long long> bits(RTS_RESID_CAP);
    RTS_CUDA_TRY(ctx, cudaMemcpy(bits.data(), ctx->d_resid + 1, sizeof(unsigned long long) * RTS_RESID_CAP,
                                 cudaMemcpyDeviceToHost));
    int rc = check_device_flag(ctx);
    if (rc != RTS_OK) return rc;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t step = ctx->solve_steps - n + i;
        memcpy(out + i, &bits[(size_t)(step % RTS_RESID_CAP)], sizeof(double));
    }
    return RTS_OK;
}

int rts_solve_residual(rts_ctx* ctx, double* residual)
{
    if (!ctx || !residual) return RTS_ERR_INVALID_ARGUMENT;
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_REQUIRE(ctx, ctx->solve_steps > 0, RTS_ERR_BAD_STATE, "rts_solve_residual before a step");
    unsigned long long bits = 0;
    const unsigned long long* slot = ctx->d_resid + 1 + ((ctx->solve_steps - 1) % RTS_RESID_CAP);
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(&bits, slot, sizeof(bits), cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    int rc = check_device_flag(ctx);
    if (rc != RTS_OK) return rc;
    memcpy(residual, &bits, sizeof(double));
    return RTS_OK;
}

int rts_solve_step(rts_ctx* ctx, int relax, double* residual)
{
    int rc = rts_solve_step_async(ctx, relax);
    if (rc != RTS_OK) return rc;
    if (residual) return rts_solve_residual(ctx, residual);
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->streams[RTS_STREAM_SCATTERING_1]));
    return RTS_OK;
}

int rts_solve_read(rts_ctx* ctx, double* S_host)
{
    if (!ctx || !S_host) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->solve_precision >= 0, RTS_ERR_BAD_STATE, "rts_solve_read before setup");
    if (ctx->solve_precision != RTS_PREC_FP64) return rts_split_read(ctx, S_host);
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(S_host, ctx->d_S, rts_bytes<double>(ctx->M * ctx->N),
                                      cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

int rts_solve_read_ibar(rts_ctx* ctx, double* ibar_host)
{
    if (!ctx || !ibar_host) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->solve_precision >= 0, RTS_ERR_BAD_STATE,
                "rts_solve_read_ibar before setup");
    if (ctx->solve_precision != RTS_PREC_FP64) return rts_split_read_ibar(ctx, ibar_host);
    // FP64 path: face mean of the device Illum, computed on the host copy.
    std::vector<double> tmp((size_t)(ctx->M * ctx->N * 4));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->streams[RTS_STREAM_SCATTERING_1]));
    RTS_CUDA_TRY(ctx, cudaMemcpy(tmp.data(), ctx->d_illum, tmp.size() * sizeof(double),
                                 cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < ctx->M * ctx->N; ++i) {
        double I = 0;
        for (int f = 0; f < 4; ++f) I += tmp[(size_t)(i * 4 + f)];
        ibar_host[i] = I / 4;
    }
    return RTS_OK;
}

int rts_synth_illum(rts_ctx* ctx, uint64_t seed, double mu, double sigma, int independent_faces)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_synth_illum before rts_init");
    rts_inputs_changed(ctx);
    return rts_launch_synth(ctx, seed, mu, sigma, independent_faces);
}

int rts_set_tuning(rts_ctx* ctx, int key, int value)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    switch (key) {
    case RTS_TUNE_FLUSH:
        RTS_REQUIRE(ctx, value >= 0 && value <= 2, RTS_ERR_INVALID_ARGUMENT,
                    "flush period %d outside [0, 2]", value);
        ctx->split_flush = value;
        return RTS_OK;
    case RTS_TUNE_SERVE_POLICY:
        RTS_REQUIRE(ctx, value >= 0 && value <= 3, RTS_ERR_INVALID_ARGUMENT, "serving policy %d not 0 to 3", value);
        ctx->serve_policy = value;
        return RTS_OK;
    case RTS_TUNE_SERVE_SLACK:
        RTS_REQUIRE(ctx, value >= 0 && value <= 100000, RTS_ERR_INVALID_ARGUMENT, "slack %d outside [0,100000]", value);
        ctx->serve_slack = value > 0 ? value : 500;
        return RTS_OK;
    case RTS_TUNE_SERVE_BUDGET:
        RTS_REQUIRE(ctx, value >= 0, RTS_ERR_INVALID_ARGUMENT, "tile budget %d below 0", value);
        ctx->serve_budget = value;
        return RTS_OK;
    case RTS_TUNE_SWEEP_CACHE:
        RTS_REQUIRE(ctx, value == 0 || value == 1, RTS_ERR_INVALID_ARGUMENT, "sweep cache switch %d not 0 or 1", value);
        ctx->sweep_cache = value;
        if (ctx->sweep) ctx->sweep->att_valid = false;
        return RTS_OK;
    case RTS_TUNE_BIAS:
        RTS_REQUIRE(ctx, value >= -1, RTS_ERR_INVALID_ARGUMENT, "bias correction %d below -1", value);
        ctx->split_bias = value;
        ctx->tuning_epoch++;  // batch tables are rebuilt at their next step or capture
        return RTS_OK;
    default:
        return rts_fail(ctx, RTS_ERR_INVALID_ARGUMENT, "unknown tuning key %d", key);
    }
}

int rts_set_precision(rts_ctx* ctx, int precision)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx,
                precision == RTS_PREC_FP64 || precision == RTS_PREC_BF16X3 || precision == RTS_PREC_FP16X3 ||
                    precision == RTS_PREC_TF32X3,
                RTS_ERR_INVALID_ARGUMENT, "rts_set_precision: unknown precision %d", precision);
    RTS_REQUIRE(ctx, precision == RTS_PREC_FP64 || ctx->cc_major == 10, RTS_ERR_UNSUPPORTED,
                "the tensor-core precisions need a Blackwell (sm_10x) device, found sm_%d%d", ctx->cc_major,
                ctx->cc_minor);
    ctx->call_precision = precision;
    return RTS_OK;
}

int rts_get_precision(const rts_ctx* ctx, int* precision)
{
    if (!ctx || !precision) return RTS_ERR_INVALID_ARGUMENT;
    *precision = ctx->call_precision;
    return RTS_OK;
}

int rts_flush_period(const rts_ctx* ctx, int precision, int* flush)
{
    if (!ctx || !flush) return RTS_ERR_INVALID_ARGUMENT;
    if (precision != RTS_PREC_BF16X3 && precision != RTS_PREC_FP16X3 && precision != RTS_PREC_TF32X3)
        return RTS_ERR_INVALID_ARGUMENT;
    *flush = rts_ctx_flush(ctx, precision);
    return RTS_OK;
}

int rts_stream_handle(rts_ctx* ctx, int stream, void** handle)
{
    if (!ctx || !handle) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, valid_stream(stream), RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    *handle = (void*)ctx->streams[stream];
    return RTS_OK;
}

int rts_launch_count(const rts_ctx* ctx, int64_t* count)
{
    if (!ctx || !count) return RTS_ERR_INVALID_ARGUMENT;
    *count = ctx->launches;
    return RTS_OK;
}

int rts_kernel_timing(rts_ctx* ctx, int enable, double* total_ms, int64_t* launches)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    double ms = 0.0;
    int64_t n = 0;
    if (enable) {
        ctx->tev_used = 0;
        ctx->timing = true;
    } else {
        for (size_t i = 0; i + 1 < ctx->tev_used; i += 2) {
            RTS_CUDA_TRY(ctx, cudaEventSynchronize(ctx->tev[i + 1]));
            float t = 0.f;
            RTS_CUDA_TRY(ctx, cudaEventElapsedTime(&t, ctx->tev[i], ctx->tev[i + 1]));
            ms += t;
            ++n;
        }
        ctx->timing = false;
    }
    if (total_ms) *total_ms = ms;
    if (launches) *launches = n;
    return RTS_OK;
}

}  // extern "C"
