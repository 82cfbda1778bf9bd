// rts_batch.cu -- public C ABI of batched problems (include/rts_scatter.h,
// "batched problems"): admission of problems with their inputs, one grouped
// launch per step, CUDA-graph capture / replay, read-back.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "rts_group.h"
#include "rts_internal.h"

namespace {

int check_desc(rts_ctx* ctx, const rts_problem_desc* d)
{
    RTS_REQUIRE(ctx, d, RTS_ERR_INVALID_ARGUMENT, "null problem descriptor");
    RTS_REQUIRE(ctx, d->N > 0 && d->M > 0 && d->groups > 0, RTS_ERR_INVALID_ARGUMENT,
                "problem sizes must be positive (N=%lld M=%lld groups=%lld)", (long long)d->N, (long long)d->M,
                (long long)d->groups);
    RTS_REQUIRE(ctx, d->M <= 65536 && d->N * d->groups <= ((int64_t)1 << 36), RTS_ERR_INVALID_ARGUMENT,
                "problem too large (M=%lld, rows=%lld)", (long long)d->M, (long long)(d->N * d->groups));
    RTS_REQUIRE(ctx, d->phase == RTS_PHASE_THOMSON || d->phase == RTS_PHASE_HG, RTS_ERR_INVALID_ARGUMENT,
                "phase must be RTS_PHASE_THOMSON or RTS_PHASE_HG");
    RTS_REQUIRE(ctx, d->phase != RTS_PHASE_HG || (d->g > -1.0 && d->g < 1.0), RTS_ERR_INVALID_ARGUMENT,
                "HG asymmetry %g outside (-1, 1)", d->g);
    RTS_REQUIRE(ctx, d->precision == RTS_PREC_FP16X3 || d->precision == RTS_PREC_BF16X3 ||
                         d->precision == RTS_PREC_TF32X3,
                RTS_ERR_INVALID_ARGUMENT,
                "batched problems run the tensor-core precisions only");
    RTS_REQUIRE(ctx, d->flush >= 0 && d->flush <= 2, RTS_ERR_INVALID_ARGUMENT, "flush %d outside [0,2]", d->flush);
    RTS_REQUIRE(ctx, d->bn == 0 || (d->bn % 16 == 0 && d->bn >= 16 && d->bn <= 256), RTS_ERR_INVALID_ARGUMENT,
                "bn %d must be a multiple of 16 in [16,256]", d->bn);
    return RTS_OK;
}

}  // namespace

extern "C" {

int rts_problem_footprint(const rts_problem_desc* desc, int64_t* bytes)
{
    if (!desc || !bytes || desc->N <= 0 || desc->M <= 0 || desc->groups <= 0) return RTS_ERR_INVALID_ARGUMENT;
    *bytes = rts_group_footprint(desc->N, desc->M, desc->groups, true, rts_split_mode(desc->precision));
    return RTS_OK;
}

int rts_batch_create(rts_ctx* ctx, rts_batch** out)
{
    if (!ctx || !out) return RTS_ERR_INVALID_ARGUMENT;
    RTS_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return rts_group_batch_new(ctx, out);
}

int rts_batch_destroy(rts_batch* batch)
{
    rts_group_batch_free(batch);
    return RTS_OK;
}

int rts_batch_add(rts_batch* batch, const rts_problem_desc* d, const float* ibar, const float* B, const double* lambda,
                  int64_t* id)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    rts_ctx* ctx = rts_group_ctx(batch);
    return rts_batch_add_on(batch, d, ibar, B, lambda, ctx->streams[RTS_STREAM_SCATTERING_1], true, id);
}

}  // extern "C"

// Set-up of a new problem queued on `st`: directions, W, split W, the Ibar
// copy and its split.  With sync the call returns once the problem is ready;
// without, the caller must see work queued on `st` finish (an event recorded
// after the call) before the problem's first step is launched on another
// stream.  Host inputs are read during the call when pageable, or by the
// queued copy when pinned (they must then stay valid until it has run).
int rts_batch_add_on(rts_batch* batch, const rts_problem_desc* d, const float* ibar, const float* B,
                     const double* lambda, cudaStream_t st, bool sync, int64_t* id)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    rts_ctx* ctx = rts_group_ctx(batch);
    int rc = check_desc(ctx, d);
    if (rc != RTS_OK) return rc;
    RTS_REQUIRE(ctx, ibar && B && lambda, RTS_ERR_INVALID_ARGUMENT, "rts_batch_add: null input");
    const int64_t N = d->N, M = d->M, G = d->groups, rows = N * G;
    for (int64_t g = 0; g < G; ++g)
        RTS_REQUIRE(ctx, lambda[g] >= 0.0 && lambda[g] <= 1.0, RTS_ERR_INVALID_ARGUMENT,
                    "albedo %g of group %lld outside [0, 1]", lambda[g], (long long)g);

    // direction set and W in scratch, followed by the FP32 Ibar staging area
    std::vector<double> xyz(3 * (size_t)M), area((size_t)M);
    double full_area = 0.0;
    rts_synth_directions(M, xyz.data(), area.data(), &full_area);
    double *d_xyz = nullptr, *d_area = nullptr;
    rc = rts_group_dirs(batch, xyz.data(), area.data(), M, &d_xyz, &d_area, st);
    if (rc != RTS_OK) return rc;
    const size_t w_bytes = (size_t)(M * M) * 8, i_bytes = (size_t)(rows * M) * 4;
    void* scratch = nullptr;
    rc = rts_group_scratch(batch, w_bytes + i_bytes, &scratch, st);
    if (rc != RTS_OK) return rc;
    double* W = static_cast<double*>(scratch);
    float* stage = reinterpret_cast<float*>(static_cast<char*>(scratch) + w_bytes);
    rc = rts_launch_weights_raw(ctx, d_xyz, d_area, (int)M, 0, (int)M, full_area, d->phase, d->g, W, st);
    if (rc != RTS_OK) return rc;

    GProb* p = nullptr;
    const int flush = d->flush > 0 ? d->flush
                                   : rts_tuned_flush(ctx, M, d->precision, N * G,
                                                     rts_auto_flush(xyz.data(), area.data(), M, full_area, 0, M,
                                                                    d->phase, d->g, d->precision));
    rc = rts_group_new_problem(batch, N, M, M, G, W, (int)M, rts_split_mode(d->precision), flush, d->bn, true, &p, st);
    if (rc != RTS_OK) return rc;
    std::vector<float> lam((size_t)G);
    for (int64_t g = 0; g < G; ++g) lam[(size_t)g] = (float)lambda[g];
    cudaError_t e = cudaMemcpyAsync(stage, ibar, i_bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->B, B, (size_t)rows * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->lam, lam.data(), (size_t)G * 4, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        int64_t tmp = 0;
        rts_group_attach(batch, p, &tmp);  // owned by the batch from here; remove frees it
        rts_group_remove_on(batch, tmp, st);
        return rts_fail(ctx, RTS_ERR_CUDA, "rts_batch_add: copy failed: %s", cudaGetErrorString(e));
    }
    rc = rts_pp_rows_from_f32(ctx, stage, N, (int)M, rows, (int)p->kpad, p->B, p->mode, p->rs, p->rows_pad, p->a[0], st,
                              p->part != nullptr);
    if (rc == RTS_OK) rc = rts_group_reset_energy(ctx, p, st);
    if (rc == RTS_OK && sync) {
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = rts_fail(ctx, RTS_ERR_CUDA, "rts_batch_add: %s", cudaGetErrorString(e));
    }
    int64_t new_id = 0;
    rts_group_attach(batch, p, &new_id);
    if (rc != RTS_OK) {
        rts_group_remove_on(batch, new_id, st);
        return rc;
    }
    if (id) *id = new_id;
    return RTS_OK;
}

extern "C" {

int rts_batch_remove(rts_batch* batch, int64_t id)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    return rts_group_remove(batch, id);
}

int rts_batch_size(rts_batch* batch, int64_t* problems, int64_t* tiles)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    if (problems) *problems = (int64_t)rts_group_count(batch);
    if (tiles) *tiles = rts_group_total_tiles(batch);
    return RTS_OK;
}

int rts_batch_step(rts_batch* batch, int relax)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    rts_ctx* ctx = rts_group_ctx(batch);
    return rts_group_step(batch, relax ? 1 : 0, ctx->streams[RTS_STREAM_SCATTERING_1]);
}

int rts_batch_capture(rts_batch* batch, int steps, int relax)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    return rts_group_capture(batch, steps, relax ? 1 : 0);
}

int rts_batch_replay(rts_batch* batch)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    return rts_group_replay(batch);
}

int rts_batch_sync(rts_batch* batch, int64_t timeout_us)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    rts_ctx* ctx = rts_group_ctx(batch);
    int rc = rts_sync_stream(ctx, RTS_STREAM_SCATTERING_1, timeout_us);
    if (rc != RTS_OK) return rc;
    int flag = 0;
    RTS_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return rts_fail(ctx, RTS_ERR_DEVICE_WAIT, "batched kernel reported device flag %d", flag);
    return RTS_OK;
}

int rts_batch_read(rts_batch* batch, int64_t id, float* S, double* residual)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    rts_ctx* ctx = rts_group_ctx(batch);
    GProb* p = rts_group_find(batch, id, nullptr);
    RTS_REQUIRE(ctx, p, RTS_ERR_INVALID_ARGUMENT, "no problem with id %lld in the batch", (long long)id);
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    if (S)
        RTS_CUDA_TRY(ctx, cudaMemcpyAsync(S, p->S32, (size_t)(p->rows * p->Mout) * 4, cudaMemcpyDeviceToHost, st));
    unsigned long long bits = 0;
    if (residual) {
        if (p->slot >= 0)
            RTS_CUDA_TRY(ctx, cudaMemcpyAsync(&bits, rts_group_resid_slot(batch, (size_t)p->slot), sizeof(bits),
                                              cudaMemcpyDeviceToHost, st));
    }
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if (residual) memcpy(residual, &bits, sizeof(double));
    int flag = 0;
    RTS_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return rts_fail(ctx, RTS_ERR_DEVICE_WAIT, "batched kernel reported device flag %d", flag);
    return RTS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// synthetic inputs generated on the device (benchmark workloads)
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ uint64_t syn_mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t syn_key(uint64_t seed, uint64_t stream)
{
    uint64_t z = seed * 0x632BE59BD9B4E019ull + stream;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double syn_uniform(uint64_t key, uint64_t idx)
{
    const uint64_t r = syn_mix64(key ^ syn_mix64(idx));
    return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// out[i] = exp(mu + sigma * normal) (lognormal) or lo + (hi-lo) * uniform,
// counter hash index i0 + i (Box-Muller on (2i, 2i+1) for the normal).
__global__ void synth_f32_kernel(float* __restrict__ out, int64_t n, uint64_t key, int64_t i0, int lognormal,
                                 double a, double b)
{
    const double two_pi = 6.283185307179586476925286766559;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t idx = (uint64_t)(i0 + i);
        if (lognormal) {
            const double u1 = syn_uniform(key, 2 * idx), u2 = syn_uniform(key, 2 * idx + 1);
            out[i] = (float)exp(a + b * (sqrt(-2.0 * log(u1)) * cos(two_pi * u2)));
        } else {
            out[i] = (float)(a + (b - a) * syn_uniform(key, idx));
        }
    }
}

int launch_synth_f32(rts_ctx* ctx, float* d_out, int64_t n, uint64_t seed, uint64_t stream, int64_t i0, int lognormal,
                     double a, double b, cudaStream_t st)
{
    int64_t blocks = (n + 255) / 256;
    if (blocks > (int64_t)ctx->num_sms * 16) blocks = (int64_t)ctx->num_sms * 16;
    if (blocks < 1) blocks = 1;
    synth_f32_kernel<<<(unsigned)blocks, 256, 0, st>>>(d_out, n, syn_key(seed, stream), i0, lognormal, a, b);
    RTS_CHECK_LAUNCH(ctx, "synth_f32_kernel");
    ctx->launches++;
    return RTS_OK;
}

}  // namespace

extern "C" int rts_batch_add_synthetic(rts_batch* batch, const rts_problem_desc* d, uint64_t seed, double mu,
                                       double sigma, double b_lo, double b_hi, const double* lambda, int64_t* id)
{
    if (!batch) return RTS_ERR_INVALID_ARGUMENT;
    rts_ctx* ctx = rts_group_ctx(batch);
    int rc = check_desc(ctx, d);
    if (rc != RTS_OK) return rc;
    RTS_REQUIRE(ctx, lambda, RTS_ERR_INVALID_ARGUMENT, "rts_batch_add_synthetic: null lambda");
    const int64_t N = d->N, M = d->M, G = d->groups, rows = N * G;
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    std::vector<double> xyz(3 * (size_t)M), area((size_t)M);
    double full_area = 0.0;
    rts_synth_directions(M, xyz.data(), area.data(), &full_area);
    double *d_xyz = nullptr, *d_area = nullptr;
    rc = rts_group_dirs(batch, xyz.data(), area.data(), M, &d_xyz, &d_area);
    if (rc != RTS_OK) return rc;
    const size_t w_bytes = (size_t)(M * M) * 8, i_bytes = (size_t)(rows * M) * 4;
    void* scratch = nullptr;
    rc = rts_group_scratch(batch, w_bytes + i_bytes, &scratch);
    if (rc != RTS_OK) return rc;
    double* W = static_cast<double*>(scratch);
    float* stage = reinterpret_cast<float*>(static_cast<char*>(scratch) + w_bytes);
    rc = rts_launch_weights_raw(ctx, d_xyz, d_area, (int)M, 0, (int)M, full_area, d->phase, d->g, W, st);
    if (rc != RTS_OK) return rc;
    GProb* p = nullptr;
    const int flush = d->flush > 0 ? d->flush
                                   : rts_tuned_flush(ctx, M, d->precision, N * G,
                                                     rts_auto_flush(xyz.data(), area.data(), M, full_area, 0, M,
                                                                    d->phase, d->g, d->precision));
    rc = rts_group_new_problem(batch, N, M, M, G, W, (int)M, rts_split_mode(d->precision), flush, d->bn, true, &p);
    if (rc != RTS_OK) return rc;
    std::vector<float> lam((size_t)G);
    for (int64_t g = 0; g < G; ++g) lam[(size_t)g] = (float)lambda[g];
    // Ibar [g][j][c]: stream 1, index (g*M + j)*N + c; B [g][c]: stream 2, index g*N + c
    rc = launch_synth_f32(ctx, stage, rows * M, seed, 1, 0, 1, mu, sigma, st);
    if (rc == RTS_OK) rc = launch_synth_f32(ctx, p->B, rows, seed, 2, 0, 0, b_lo, b_hi, st);
    cudaError_t e = cudaSuccess;
    if (rc == RTS_OK) e = cudaMemcpyAsync(p->lam, lam.data(), (size_t)G * 4, cudaMemcpyHostToDevice, st);
    if (rc == RTS_OK && e == cudaSuccess)
        rc = rts_pp_rows_from_f32(ctx, stage, N, (int)M, rows, (int)p->kpad, p->B, p->mode, p->rs, p->rows_pad,
                                  p->a[0], st, p->part != nullptr);
    if (rc == RTS_OK && e == cudaSuccess) rc = rts_group_reset_energy(ctx, p, st);
    if (rc == RTS_OK && e == cudaSuccess) e = cudaStreamSynchronize(st);
    int64_t new_id = 0;
    rts_group_attach(batch, p, &new_id);
    if (rc != RTS_OK || e != cudaSuccess) {
        rts_group_remove(batch, new_id);
        return rc != RTS_OK ? rc : rts_fail(ctx, RTS_ERR_CUDA, "rts_batch_add_synthetic: %s", cudaGetErrorString(e));
    }
    if (id) *id = new_id;
    return RTS_OK;
}

extern "C" int rts_synth_host_f32(rts_ctx* ctx, uint64_t seed, uint64_t stream, int lognormal, double a, double b,
                                  int64_t i0, int64_t n, float* host_out)
{
    if (!ctx || n < 0 || (n > 0 && !host_out)) return RTS_ERR_INVALID_ARGUMENT;
    if (n == 0) return RTS_OK;
    const int64_t chunk = std::min<int64_t>(n, (int64_t)1 << 26);
    void* tmp = nullptr;
    int rc = rts_dmalloc(ctx, &tmp, (size_t)chunk * 4, "synthetic staging");
    if (rc != RTS_OK) return rc;
    cudaStream_t st = ctx->streams[RTS_STREAM_PARAMS];
    for (int64_t off = 0; off < n && rc == RTS_OK; off += chunk) {
        const int64_t m = std::min(chunk, n - off);
        rc = launch_synth_f32(ctx, static_cast<float*>(tmp), m, seed, stream, i0 + off, lognormal, a, b, st);
        if (rc == RTS_OK &&
            (cudaMemcpyAsync(host_out + off, tmp, (size_t)m * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
             cudaStreamSynchronize(st) != cudaSuccess))
            rc = rts_fail(ctx, RTS_ERR_CUDA, "rts_synth_host_f32: copy failed");
    }
    rts_dfree(ctx, tmp, (size_t)chunk * 4);
    return rc;
}
