// rts_split.cu -- the context's split-precision (tcgen05) entry points:
// the resident source iteration (rts_solve_* with FP16x3 / BF16x3) and the
// host-buffer call rts_scattering_update.  Both run the persistent grouped
// kernel of rts_group.cu on a private one-problem batch whose A rows come
// from the reference's face-layout Illum on the device and whose W is the
// context's FP64 direction-pair matrix (Thomson, HG or caller-supplied).
//
// Reference counterpart: d_GetS_MPI_Stream (cuda/cuda_kernel.cu:82-111) and
// its launch in CalculateIntScatteringAsyncMPIStream (cuda/cuda_solve.cu:89-111).
#include <cstring>

#include "rts_group.h"
#include "rts_internal.h"

namespace {

// (Re)build the one-problem batch `*pb` from the context's current Illum and W.
int build_problem(rts_ctx* ctx, rts_batch** pb, int64_t* id, int precision, bool iterative, const double* B_dev,
                  double lambda, double* S64, cudaStream_t st)
{
    const bool fp16 = precision == RTS_PREC_FP16X3;
    const int64_t N = ctx->N, Min = ctx->M, Mout = ctx->local();
    const int flush = ctx->split_flush > 0 ? ctx->split_flush : 1;
    GProb* p = nullptr;
    if (*pb) {
        p = rts_group_find(*pb, *id, nullptr);
        if (p && (p->fp16 != fp16 || p->N != N || p->M != Min || p->Mout != Mout || (iterative && !p->a[1]) ||
                  p->flush != flush)) {
            int rc = rts_group_remove(*pb, *id);
            if (rc != RTS_OK) return rc;
            p = nullptr;
        }
    } else {
        int rc = rts_group_batch_new(ctx, pb);
        if (rc != RTS_OK) return rc;
    }
    if (!p) {
        int rc = rts_group_new_problem(*pb, N, Min, Mout, 1, ctx->d_W, (int)Mout, fp16, flush, 0, iterative, &p);
        if (rc != RTS_OK) return rc;
        rc = rts_group_attach(*pb, p, id);
        if (rc != RTS_OK) return rc;
    } else {
        // W may have changed (phase / custom weights): split it again
        int rc = rts_pp_split_w(ctx, ctx->d_W, (int)Min, (int)Mout, (int)Mout, (int)p->kpad, (int)p->mpad, fp16, p->wc,
                                p->cs, st);
        if (rc != RTS_OK) return rc;
    }
    p->cur = 0;
    p->S64 = S64;
    p->use_B = B_dev != nullptr;
    int rc = rts_pp_rows_from_faces(ctx, ctx->d_illum, N, (int)Min, (int)p->kpad, B_dev, fp16, p->rs, p->rows_pad,
                                    p->a[0], st);
    if (rc != RTS_OK) return rc;
    if (B_dev) {
        rc = rts_pp_f64_to_f32(ctx, B_dev, p->B, N, st);
        if (rc != RTS_OK) return rc;
    }
    const float lam = (float)lambda;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(p->lam, &lam, sizeof(float), cudaMemcpyHostToDevice, st));
    if (p->S32) RTS_CUDA_TRY(ctx, cudaMemsetAsync(p->S32, 0, (size_t)(p->rows * p->Mout * 4), st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // the host lambda must outlive its copy
    rts_group_invalidate(*pb);  // the batch table caches cur / S64 / use_B
    return RTS_OK;
}

}  // namespace

int rts_split_setup(rts_ctx* ctx, int precision)
{
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED,
                "the tensor-core path needs a Blackwell (sm_10x) device, found sm_%d%d", ctx->cc_major, ctx->cc_minor);
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), st));
    int rc = build_problem(ctx, &ctx->split.iter, &ctx->split.iter_id, precision, true, ctx->d_B, ctx->solve_lambda,
                           nullptr, st);
    if (rc != RTS_OK) return rc;
    ctx->split.precision = precision;
    return RTS_OK;
}

int rts_split_step(rts_ctx* ctx, bool relax, cudaStream_t st)
{
    RTS_REQUIRE(ctx, ctx->split.iter, RTS_ERR_BAD_STATE, "no tensor-path source iteration set up");
    RTS_REQUIRE(ctx, !relax || ctx->local() == ctx->M, RTS_ERR_UNSUPPORTED, "relaxation needs all out-directions local");
    int rc = rts_group_step(ctx->split.iter, relax ? 1 : 0, st);
    if (rc != RTS_OK) return rc;
    // the step's residual into the context's ring slot
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->resid_target, rts_group_resid_slot(ctx->split.iter, 0),
                                      sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
    return RTS_OK;
}

int rts_split_oneshot(rts_ctx* ctx, int precision, const double* B, double lambda, cudaStream_t st)
{
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED, "the tensor-core path needs a Blackwell (sm_10x) device");
    int rc = build_problem(ctx, &ctx->split.shot, &ctx->split.shot_id, precision, false, B, lambda, ctx->d_S, st);
    if (rc != RTS_OK) return rc;
    ctx->split.shot_precision = precision;
    return rts_group_step(ctx->split.shot, 0, st);
}

int rts_split_read(rts_ctx* ctx, double* S_host)
{
    RTS_REQUIRE(ctx, ctx->split.iter, RTS_ERR_BAD_STATE, "no tensor-path source iteration set up");
    GProb* p = rts_group_find(ctx->split.iter, ctx->split.iter_id, nullptr);
    RTS_REQUIRE(ctx, p && p->S32, RTS_ERR_BAD_STATE, "tensor-path problem missing");
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    const int64_t n = p->Mout * p->N;
    int rc = rts_pp_f32_to_f64(ctx, p->S32, ctx->d_S, n, st);  // d_S is free scratch on this path
    if (rc != RTS_OK) return rc;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(S_host, ctx->d_S, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    int flag = 0;
    RTS_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return rts_fail(ctx, RTS_ERR_DEVICE_WAIT, "tensor-path kernel reported device flag %d", flag);
    return RTS_OK;
}

int rts_split_read_ibar(rts_ctx* ctx, double* ibar_host)
{
    RTS_REQUIRE(ctx, ctx->split.iter, RTS_ERR_BAD_STATE, "no tensor-path operands set up");
    GProb* p = rts_group_find(ctx->split.iter, ctx->split.iter_id, nullptr);
    RTS_REQUIRE(ctx, p, RTS_ERR_BAD_STATE, "tensor-path problem missing");
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    const int64_t n = p->M * p->N;
    int rc = rts_pp_join_rows(ctx, p->a[p->cur], p->N, (int)p->M, p->rows, (int)p->kpad,
                              p->fp16 ? p->rs + p->rows_pad : nullptr, p->fp16, ctx->d_S, st);
    if (rc != RTS_OK) return rc;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ibar_host, ctx->d_S, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

void rts_split_free(rts_ctx* ctx)
{
    rts_group_batch_free(ctx->split.iter);
    rts_group_batch_free(ctx->split.shot);
    ctx->split = rts_split_state();
}
