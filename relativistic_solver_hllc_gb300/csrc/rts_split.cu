// rts_split.cu -- the context's split-precision (tcgen05) entry points:
// the resident source iteration (rts_solve_* with FP16x3 / BF16x3) and the
// host-buffer call rts_scattering_update.  Both run the persistent grouped
// kernel of rts_group.cu on a private one-problem batch whose A rows come
// from the reference's face-layout Illum on the device and whose W is the
// context's FP64 direction-pair matrix (Thomson, HG or caller-supplied).
//
// Reference counterpart: d_GetS_MPI_Stream (cuda/cuda_kernel.cu:82-111) and
// its launch in CalculateIntScatteringAsyncMPIStream (cuda/cuda_solve.cu:89-111).
#include <algorithm>
#include <cstring>

#include "rts_group.h"
#include "rts_internal.h"

int rts_ctx_flush(const rts_ctx* ctx, int precision)
{
    if (ctx->split_flush > 0) return ctx->split_flush;
    const int cap = rts_auto_flush(ctx->h_xyz.data(), ctx->h_area.data(), ctx->M, ctx->full_area, ctx->out_start,
                                   ctx->out_end, ctx->phase, ctx->phase_g, precision);
    return rts_tuned_flush(ctx, ctx->M, precision, ctx->N, cap);
}

namespace {

// (Re)build the one-problem batch `*pb` from the context's current Illum and W.
int build_problem(rts_ctx* ctx, rts_batch** pb, int64_t* id, int precision, bool iterative, const double* B_dev,
                  double lambda, double* S64, cudaStream_t st)
{
    const int mode = rts_split_mode(precision);
    const int64_t N = ctx->N, Min = ctx->M, Mout = ctx->local();
    const int flush = rts_ctx_flush(ctx, precision);
    GProb* p = nullptr;
    if (*pb) {
        p = rts_group_find(*pb, *id, nullptr);
        if (p && (p->mode != mode || p->N != N || p->M != Min || p->Mout != Mout || (iterative && !p->a[1]) ||
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
        int rc = rts_group_new_problem(*pb, N, Min, Mout, 1, ctx->d_W, (int)Mout, mode, flush, 0, iterative, &p);
        if (rc != RTS_OK) return rc;
        rc = rts_group_attach(*pb, p, id);
        if (rc != RTS_OK) return rc;
    } else {
        // W may have changed (phase / custom weights): split it again, with
        // the correction's statistics
        int rc = rts_group_set_w(ctx, p, ctx->d_W, (int)Mout, st);
        if (rc != RTS_OK) return rc;
    }
    p->cur = 0;
    p->S64 = S64;
    p->use_B = B_dev != nullptr;
    // once per set-up: the direct preparation, which needs no staging
    int rc = rts_pp_rows_from_faces(ctx, ctx->d_illum, N, N, (int)Min, (int)p->kpad, B_dev, mode, p->rs, p->rows_pad,
                                    p->a[0], st, p->part != nullptr);
    if (rc != RTS_OK) return rc;
    if (B_dev) {
        rc = rts_pp_f64_to_f32(ctx, B_dev, p->B, N, st);
        if (rc != RTS_OK) return rc;
    }
    const float lam = (float)lambda;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(p->lam, &lam, sizeof(float), cudaMemcpyHostToDevice, st));
    if (p->S32) RTS_CUDA_TRY(ctx, cudaMemsetAsync(p->S32, 0, (size_t)(p->rows * p->Mout * 4), st));
    rc = rts_group_reset_energy(ctx, p, st);  // the restarted iteration's first step is uncorrected
    if (rc != RTS_OK) return rc;
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

namespace {

int ensure_pipeline(rts_ctx* ctx)
{
    rts_split_state& s = ctx->split;
    if (s.copy_in) return RTS_OK;
    RTS_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&s.copy_in, cudaStreamNonBlocking));
    RTS_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&s.copy_out, cudaStreamNonBlocking));
    RTS_CUDA_TRY(ctx, cudaEventCreateWithFlags(&s.ev_start, cudaEventDisableTiming));
    for (int i = 0; i < RTS_HOST_CHUNKS; ++i) {
        RTS_CUDA_TRY(ctx, cudaEventCreateWithFlags(&s.ev_in[i], cudaEventDisableTiming));
        RTS_CUDA_TRY(ctx, cudaEventCreateWithFlags(&s.ev_done[i], cudaEventDisableTiming));
    }
    return RTS_OK;
}

// The one-problem batch of cell range i with n cells, rebuilt when its shape,
// precision or flush period changed; W split again when the context's W did.
int chunk_problem(rts_ctx* ctx, int i, int64_t n, int mode, int flush, GProb** out, cudaStream_t st)
{
    rts_split_state& s = ctx->split;
    const int64_t M = ctx->M, Mout = ctx->local();
    int rc;
    GProb* p = s.chunk[i] ? rts_group_find(s.chunk[i], s.chunk_id[i], nullptr) : nullptr;
    if (p && (p->mode != mode || p->N != n || p->M != M || p->Mout != Mout || p->flush != flush)) {
        if ((rc = rts_group_remove(s.chunk[i], s.chunk_id[i])) != RTS_OK) return rc;
        p = nullptr;
    }
    if (!s.chunk[i] && (rc = rts_group_batch_new(ctx, &s.chunk[i])) != RTS_OK) return rc;
    if (!p) {
        rc = rts_group_new_problem(s.chunk[i], n, M, Mout, 1, ctx->d_W, (int)Mout, mode, flush, 0, false, &p);
        if (rc != RTS_OK) return rc;
        if ((rc = rts_group_attach(s.chunk[i], p, &s.chunk_id[i])) != RTS_OK) return rc;
        s.chunk_w_version[i] = ctx->w_version;
    } else if (s.chunk_w_version[i] != ctx->w_version) {
        rc = rts_pp_split_w(ctx, ctx->d_W, (int)M, (int)Mout, (int)Mout, (int)p->kpad, (int)p->mpad, mode, p->wc, p->cs,
                            st);
        if (rc != RTS_OK) return rc;
        s.chunk_w_version[i] = ctx->w_version;
    }
    *out = p;
    return RTS_OK;
}

}  // namespace

// rts_scattering_update at FP16x3 / BF16x3, pipelined over cell ranges.
// Row c of S depends only on row c of Ibar, so the N cells are cut into up
// to RTS_HOST_CHUNKS ranges; range i is copied in (one strided 2-D copy of
// its columns of the [M][N][4] host Illum), split and contracted on the
// scattering stream, and copied out (strided 2-D copy of its columns of the
// [local][N] S), so the H2D of one range, the compute of the previous one
// and the D2H of the one before run at the same time.  The device copy of
// Illum ends up complete, as after the reference's CalculateIntScattering.
int rts_split_host_call(rts_ctx* ctx, int precision, const double* illum_host, const double* B_host, double lambda,
                        double* S_host)
{
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED, "the tensor-core path needs a Blackwell (sm_10x) device");
    int rc = ensure_pipeline(ctx);
    if (rc != RTS_OK) return rc;
    rts_split_state& s = ctx->split;
    const int mode = rts_split_mode(precision);
    const bool update = B_host != nullptr && lambda != 1.0;
    const int64_t N = ctx->N, M = ctx->M, Mout = ctx->local();
    const int flush = rts_ctx_flush(ctx, precision);
    const int64_t tiles = (N + 127) / 128;
    const int nch = (int)std::min<int64_t>(RTS_HOST_CHUNKS, tiles);
    const int64_t csz = (tiles + nch - 1) / nch * 128;  // cells per range, whole 128-cell tiles
    cudaStream_t sc = ctx->streams[RTS_STREAM_SCATTERING_1];
    const float lamf = (float)lambda;

    // set-up (host-synchronous, before any copy is queued)
    GProb* probs[RTS_HOST_CHUNKS] = {};
    int used = 0;
    for (int i = 0; i < nch; ++i) {
        const int64_t c0 = i * csz, n = std::min(N, c0 + csz) - c0;
        if (n <= 0) break;
        GProb* p = nullptr;
        if ((rc = chunk_problem(ctx, i, n, mode, flush, &p, sc)) != RTS_OK) return rc;
        const bool changed = p->S64 != ctx->d_S + c0 || p->ldS != N || p->use_B != update || p->cur != 0;
        p->cur = 0;
        p->S64 = ctx->d_S + c0;
        p->ldS = N;
        p->use_B = update;
        if (update) RTS_CUDA_TRY(ctx, cudaMemcpyAsync(p->lam, &lamf, sizeof(float), cudaMemcpyHostToDevice, sc));
        if (changed) rts_group_invalidate(s.chunk[i]);
        if ((rc = rts_group_prepare(s.chunk[i], 0, sc)) != RTS_OK) return rc;
        probs[used++] = p;
    }
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(sc));  // the host lambda must outlive its copies

    auto drain = [&]() {
        cudaStreamSynchronize(s.copy_in);
        cudaStreamSynchronize(sc);
        cudaStreamSynchronize(s.copy_out);
    };
    RTS_CUDA_TRY(ctx, cudaEventRecord(s.ev_start, sc));
    RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(s.copy_in, s.ev_start, 0));
    RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(s.copy_out, s.ev_start, 0));
    for (int i = 0; i < used && rc == RTS_OK; ++i) {
        GProb* p = probs[i];
        const int64_t c0 = i * csz, n = p->N;
        cudaError_t e = cudaMemcpy2DAsync(ctx->d_illum + c0 * 4, (size_t)N * 32, illum_host + c0 * 4, (size_t)N * 32,
                                          (size_t)n * 32, (size_t)M, cudaMemcpyHostToDevice, s.copy_in);
        if (e == cudaSuccess && update)
            e = cudaMemcpyAsync(ctx->d_B + c0, B_host + c0, (size_t)n * 8, cudaMemcpyHostToDevice, s.copy_in);
        if (e == cudaSuccess) e = cudaEventRecord(s.ev_in[i], s.copy_in);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sc, s.ev_in[i], 0);
        if (e != cudaSuccess) {
            rc = rts_fail(ctx, RTS_ERR_CUDA, "host-call copy in: %s", cudaGetErrorString(e));
            break;
        }
        rc = rts_pp_rows_from_faces(ctx, ctx->d_illum + c0 * 4, n, N, (int)M, (int)p->kpad,
                                    update ? ctx->d_B + c0 : nullptr, mode, p->rs, p->rows_pad, p->a[0], sc);
        if (rc == RTS_OK && update) rc = rts_pp_f64_to_f32(ctx, ctx->d_B + c0, p->B, n, sc);
        if (rc == RTS_OK) rc = rts_group_step(s.chunk[i], 0, sc);
        if (rc != RTS_OK) break;
        e = cudaEventRecord(s.ev_done[i], sc);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s.copy_out, s.ev_done[i], 0);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(S_host + c0, (size_t)N * 8, ctx->d_S + c0, (size_t)N * 8, (size_t)n * 8,
                                  (size_t)Mout, cudaMemcpyDeviceToHost, s.copy_out);
        if (e != cudaSuccess) rc = rts_fail(ctx, RTS_ERR_CUDA, "host-call copy out: %s", cudaGetErrorString(e));
    }
    drain();
    if (rc != RTS_OK) return rc;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return rts_fail(ctx, RTS_ERR_CUDA, "host call: %s", cudaGetErrorString(e));
    int flag = 0;
    RTS_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return rts_fail(ctx, RTS_ERR_DEVICE_WAIT, "tensor-path kernel reported device flag %d", flag);
    return RTS_OK;
}

// On the device Illum and into the device S, all on `st` (no copies, no host
// synchronisation): one cell range over all cells -- with nothing to copy,
// the host-buffer call's ranges would only multiply the launches.  The
// range's problem is the host-buffer call's first (rebuilt when the call
// alternates with host-buffer calls).
static int ensure_staging(rts_ctx* ctx);
static bool no_room(int rc);
static int record_on(rts_ctx* ctx, cudaEvent_t& ev, cudaStream_t st);

// Rows of cells [0, n) of a device Illum whose rows hold `ld` cells into A and
// rs on `st`: the staged preparation in the integral calls' staging (waiting
// for their preparation and face sums in flight, and leaving them to prepare
// their own rows again), or, without room for the staging, the direct one.
// The two give the same rows bit for bit.
static int prepare_device_rows(rts_ctx* ctx, const double* illum, int64_t n, int64_t ld, int M, int kpad,
                               const double* B, int mode, float* rs, int64_t npad, uint16_t* A, cudaStream_t st,
                               bool bound)
{
    rts_split_state& s = ctx->split;
    int rc = ensure_staging(ctx);
    if (rc != RTS_OK) {
        if (!no_room(rc)) return rc;
        return rts_pp_rows_from_faces(ctx, illum, n, ld, M, kpad, B, mode, rs, npad, A, st, bound);
    }
    if (s.ev_prep) RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(st, s.ev_prep, 0));
    if (s.ev_eager) RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(st, s.ev_eager, 0));
    s.call_version = -1;
    s.eager_next = -1;
    rc = rts_pp_rows_from_faces_staged(ctx, illum, n, ld, M, kpad, B, mode, rs, npad, A, s.call_sums, s.call_max, st,
                                       bound);
    if (rc == RTS_OK) rc = record_on(ctx, s.ev_prep, st);  // later users of the staging wait for this one
    return rc;
}

// The scattering integral of the device Illum into the FP64 device S (all
// out-directions), on `st`, for the on-device source iteration.  The rows
// come from the staged preparation (one read of the Illum into FP64 face
// sums and per-cell maxima, then scales and split on the integer pipe), bit
// for bit the rows of the direct one.  Its staging is the asynchronous
// calls': it waits for their preparation and face sums in flight, and leaves
// them to prepare their rows again.  Without room for the staging (HBM
// budget or memory) the rows are prepared directly.
int rts_split_device_call(rts_ctx* ctx, int precision, cudaStream_t st)
{
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED, "the tensor-core path needs a Blackwell (sm_10x) device");
    rts_split_state& s = ctx->split;
    const int mode = rts_split_mode(precision);
    const int64_t N = ctx->N, M = ctx->M;
    const int flush = rts_ctx_flush(ctx, precision);
    const int nch = 1;
    const int64_t csz = N;
    int rc;
    for (int i = 0; i < nch; ++i) {
        const int64_t c0 = i * csz, n = std::min(N, c0 + csz) - c0;
        if (n <= 0) break;
        GProb* p = nullptr;
        if ((rc = chunk_problem(ctx, i, n, mode, flush, &p, st)) != RTS_OK) return rc;
        const bool changed = p->S64 != ctx->d_S + c0 || p->ldS != N || p->use_B || p->cur != 0;
        p->cur = 0;
        p->S64 = ctx->d_S + c0;
        p->ldS = N;
        p->use_B = false;
        if (changed) rts_group_invalidate(s.chunk[i]);
        if ((rc = rts_group_prepare(s.chunk[i], 0, st)) != RTS_OK) return rc;
        rc = prepare_device_rows(ctx, ctx->d_illum + c0 * 4, n, N, (int)M, (int)p->kpad, nullptr, mode, p->rs,
                                 p->rows_pad, p->a[0], st, false);
        if (rc == RTS_OK) rc = rts_group_step(s.chunk[i], 0, st);
        if (rc != RTS_OK) return rc;
    }
    return RTS_OK;
}

// rts_scattering_async at a tensor precision (rts_split_async below): local
// out-directions [start, end) of the device Illum into rows [start, end) of
// the FP64 device S, on `st`.  Stream slot `slot` keeps its own one-problem
// batch (the split W columns [start, end), table, residual), rebuilt when the
// range, shape, precision or flush period changes and its W split again when
// the context's W changed.  The split Ibar rows and their row scales depend
// on the Illum only and are shared by the slots: a call prepares them, and
// the next call on each other slot waits on that preparation's event and
// reads them.  Two calls queued on different slots at once -- the
// reference's pair [0, size_1) on scattering stream 1 and [0, local) on
// scattering stream 2 -- therefore write no common buffer except the rows of
// S they share, into which both write the same values (each output's
// arithmetic does not depend on the tiling of the out-directions).  After the
// first call of a slot nothing synchronises the host.
//
// Frees the shared split Ibar rows and the staging (cudaFree waits for the
// device, so no contraction still reads them).
static void free_call_rows(rts_ctx* ctx)
{
    rts_split_state& s = ctx->split;
    rts_dfree(ctx, s.call_a, s.call_a_bytes);
    rts_dfree(ctx, s.call_rs, s.call_rs_bytes);
    rts_dfree(ctx, s.call_sums, s.call_sums_bytes);
    rts_dfree(ctx, s.call_max, s.call_max_bytes);
    s.call_a = nullptr;
    s.call_rs = nullptr;
    s.call_sums = nullptr;
    s.call_max = nullptr;
    s.call_a_bytes = s.call_rs_bytes = s.call_sums_bytes = s.call_max_bytes = 0;
    s.call_mode = -1;
    s.call_N = s.call_M = 0;
    s.call_gen++;
    s.call_version = -1;
    s.prep_slot = -1;
    s.eager_next = -1;
}

// The shared rows for (N, M, mode): allocated on first use and when the
// precision or the sizes change (the slots' problems, whose tensor maps hold
// the old address, are rebuilt: slot_gen).
// The staging of the staged preparation: FP64 face sums [M][N] and per-cell
// maxima [N].  When it does not fit (RTS_ERR_OVER_BUDGET or
// RTS_ERR_OUT_OF_MEMORY) it stays absent and the callers prepare the rows
// directly from the faces, which gives the same rows bit for bit.
static int ensure_staging(rts_ctx* ctx)
{
    rts_split_state& s = ctx->split;
    const size_t ibytes = (size_t)(ctx->M * ctx->N * 8), mbytes = (size_t)(ctx->N * 8);
    if (s.call_sums && s.call_sums_bytes == ibytes && s.call_max_bytes == mbytes) return RTS_OK;
    rts_dfree(ctx, s.call_sums, s.call_sums_bytes);  // cudaFree waits for the device
    rts_dfree(ctx, s.call_max, s.call_max_bytes);
    s.call_sums = nullptr;
    s.call_max = nullptr;
    s.call_sums_bytes = s.call_max_bytes = 0;
    s.eager_next = -1;
    void *ib = nullptr, *mx = nullptr;
    int rc = rts_dmalloc(ctx, &ib, ibytes, "FP64 face sums (staging)");
    if (rc == RTS_OK) rc = rts_dmalloc(ctx, &mx, mbytes, "per-cell maxima (staging)");
    if (rc != RTS_OK) {
        rts_dfree(ctx, ib, ib ? ibytes : 0);
        return rc;
    }
    s.call_sums = (double*)ib;
    s.call_max = (unsigned long long*)mx;
    s.call_sums_bytes = ibytes;
    s.call_max_bytes = mbytes;
    return RTS_OK;
}

static bool no_room(int rc) { return rc == RTS_ERR_OVER_BUDGET || rc == RTS_ERR_OUT_OF_MEMORY; }

static int ensure_call_rows(rts_ctx* ctx, int mode, int64_t rows_pad, int64_t units)
{
    rts_split_state& s = ctx->split;
    if (s.call_a && s.call_mode == mode && s.call_N == ctx->N && s.call_M == ctx->M) return RTS_OK;
    free_call_rows(ctx);
    const size_t abytes = (size_t)(rows_pad * units * 2), rbytes = (size_t)(2 * rows_pad * 4);
    void *a = nullptr, *r = nullptr;
    int rc = rts_dmalloc(ctx, &a, abytes, "split Ibar rows of the integral calls");
    if (rc == RTS_OK) rc = rts_dmalloc(ctx, &r, rbytes, "row scales of the integral calls");
    s.call_a = (uint16_t*)a;
    s.call_rs = (float*)r;
    s.call_a_bytes = a ? abytes : 0;
    s.call_rs_bytes = r ? rbytes : 0;
    if (rc == RTS_OK && cudaMemset(a, 0, abytes) != cudaSuccess)  // padding rows stay zero
        rc = rts_fail(ctx, RTS_ERR_CUDA, "clearing the shared split rows failed");
    // the staging is optional: without room for it the calls prepare directly
    if (rc == RTS_OK && (rc = ensure_staging(ctx)) != RTS_OK && no_room(rc)) rc = RTS_OK;
    if (rc != RTS_OK) {
        free_call_rows(ctx);
        return rc;
    }
    s.call_mode = mode;
    s.call_N = ctx->N;
    s.call_M = ctx->M;
    return RTS_OK;
}

static int record_on(rts_ctx* ctx, cudaEvent_t& ev, cudaStream_t st)
{
    if (!ev) RTS_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    RTS_CUDA_TRY(ctx, cudaEventRecord(ev, st));
    return RTS_OK;
}

int rts_split_eager_send(rts_ctx* ctx, int64_t shift_dev, int64_t size)
{
    rts_split_state& s = ctx->split;
    if (ctx->cc_major != 10) return RTS_OK;
    const int64_t per = 4 * ctx->N, M = ctx->M;
    const int mode = rts_split_mode(ctx->call_precision);
    const int64_t j0 = shift_dev / per, j1 = (shift_dev + size) / per;
    const bool whole = size > 0 && shift_dev % per == 0 && size % per == 0 && j1 <= M;
    // a sequence runs from direction 0, each direction once and in order,
    // with nothing else written in between (the copy itself bumped the version)
    const bool next = whole && j0 > 0 && j0 == s.eager_next && s.eager_mode == mode &&
                      s.eager_version == ctx->inputs_version - 1;
    if (!whole || (j0 != 0 && !next)) {
        s.eager_next = -1;  // this Illum is prepared whole at the call
        return RTS_OK;
    }
    int bn, n_tiles;
    int64_t kpad, mpad, rows_pad, m_tiles;
    rts_group_geometry(M, M, ctx->N, 0, &bn, &n_tiles, &kpad, &mpad, &rows_pad, &m_tiles);
    int rc = ensure_call_rows(ctx, mode, rows_pad, (mode == 2 ? 4 : 2) * kpad);
    if (rc != RTS_OK) return rc;
    if (!s.call_sums) {  // no staging: this Illum is prepared directly at the call
        s.eager_next = -1;
        return RTS_OK;
    }
    if (!s.eager_st) RTS_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&s.eager_st, cudaStreamNonBlocking));
    cudaStream_t s1 = ctx->streams[RTS_STREAM_SCATTERING_1];
    if (j0 == 0) {
        // a new sequence: the staging may still be read by a preparation or
        // contraction queued before
        if (s.ev_prep) RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(s.eager_st, s.ev_prep, 0));
        for (int i = 0; i < RTS_STREAM_COUNT; ++i)
            if (s.use_recorded[i]) RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(s.eager_st, s.ev_use[i], 0));
        if (mode == 1)
            RTS_CUDA_TRY(ctx, cudaMemsetAsync(s.call_max, 0, (size_t)ctx->N * sizeof(unsigned long long), s.eager_st));
    }
    if ((rc = record_on(ctx, s.ev_sent, s1)) != RTS_OK) return rc;
    RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(s.eager_st, s.ev_sent, 0));
    rc = rts_pp_face_sums(ctx, ctx->d_illum, ctx->N, ctx->N, (int)j0, (int)j1, s.call_sums,
                          mode == 1 ? s.call_max : nullptr, s.eager_st);
    if (rc == RTS_OK) rc = record_on(ctx, s.ev_eager, s.eager_st);
    if (rc != RTS_OK) {
        s.eager_next = -1;
        return rc;
    }
    s.eager_next = j1;
    s.eager_mode = mode;
    s.eager_version = ctx->inputs_version;
    return RTS_OK;
}

int rts_split_async(rts_ctx* ctx, int precision, int64_t start, int64_t end, int slot, cudaStream_t st)
{
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED, "the tensor-core path needs a Blackwell (sm_10x) device");
    RTS_REQUIRE(ctx, slot >= 0 && slot < RTS_STREAM_COUNT, RTS_ERR_INVALID_ARGUMENT, "bad stream slot %d", slot);
    rts_split_state& s = ctx->split;
    const int mode = rts_split_mode(precision);
    const int64_t N = ctx->N, M = ctx->M, loc = ctx->local(), Mout = end - start;
    const int flush = rts_ctx_flush(ctx, precision);
    int bn, n_tiles;
    int64_t kpad, mpad, rows_pad, m_tiles;
    rts_group_geometry(M, Mout, N, 0, &bn, &n_tiles, &kpad, &mpad, &rows_pad, &m_tiles);
    int rc = ensure_call_rows(ctx, mode, rows_pad, (mode == 2 ? 4 : 2) * kpad);
    if (rc != RTS_OK) return rc;
    GProb* p = s.slot[slot] ? rts_group_find(s.slot[slot], s.slot_id[slot], nullptr) : nullptr;
    if (p && (p->mode != mode || p->N != N || p->M != M || p->Mout != Mout || p->flush != flush ||
              s.slot_start[slot] != start || s.slot_gen[slot] != s.call_gen)) {
        if ((rc = rts_group_remove_on(s.slot[slot], s.slot_id[slot], st)) != RTS_OK) return rc;
        p = nullptr;
    }
    if (!s.slot[slot] && (rc = rts_group_batch_new(ctx, &s.slot[slot])) != RTS_OK) return rc;
    if (!p) {
        rc = rts_group_new_problem(s.slot[slot], N, M, Mout, 1, ctx->d_W + start, (int)loc, mode, flush, 0, false, &p,
                                   st, s.call_a, s.call_rs);
        if (rc != RTS_OK) return rc;
        if ((rc = rts_group_attach(s.slot[slot], p, &s.slot_id[slot])) != RTS_OK) return rc;
        s.slot_start[slot] = start;
        s.slot_w_version[slot] = ctx->w_version;
        s.slot_gen[slot] = s.call_gen;
    } else if (s.slot_w_version[slot] != ctx->w_version) {
        rc = rts_pp_split_w(ctx, ctx->d_W + start, (int)M, (int)Mout, (int)loc, (int)p->kpad, (int)p->mpad, mode, p->wc,
                            p->cs, st);
        if (rc != RTS_OK) return rc;
        s.slot_w_version[slot] = ctx->w_version;
    }
    double* const S64 = ctx->d_S + start * N;
    if (p->S64 != S64 || p->ldS != N || p->use_B || p->cur != 0) {
        p->cur = 0;
        p->S64 = S64;
        p->ldS = N;
        p->use_B = false;
        rts_group_invalidate(s.slot[slot]);
    }
    // The split Ibar rows depend on the Illum only.  A call prepares them;
    // the next call on each other slot reuses them while the inputs are
    // unchanged (the reference's pair of calls on scattering streams 1 and 2
    // reads one Illum); any call on the preparing slot prepares them again,
    // so Illum written through the device pointers between the pairs is seen.
    const bool reuse = s.call_version == ctx->inputs_version && s.prep_slot >= 0 && s.prep_slot != slot &&
                       !s.prep_served[slot];
    if (reuse) {
        RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(st, s.ev_prep, 0));
        s.prep_served[slot] = true;
    } else {
        // the rows and the staging may still be read by contractions queued
        // on the other slots, and the staging written by face sums in flight
        for (int i = 0; i < RTS_STREAM_COUNT; ++i)
            if (i != slot && s.use_recorded[i]) RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(st, s.ev_use[i], 0));
        if (s.ev_eager) RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(st, s.ev_eager, 0));
        // and the staging by the device source iteration's preparation
        if (s.ev_prep) RTS_CUDA_TRY(ctx, cudaStreamWaitEvent(st, s.ev_prep, 0));
        s.call_version = -1;
        // the face sums of this Illum, when its copies summed every direction
        const bool eager = s.call_sums && s.eager_next == M && s.eager_mode == mode &&
                           s.eager_version == ctx->inputs_version;
        if (eager)
            rc = rts_pp_rows_from_sums(ctx, N, (int)M, (int)kpad, nullptr, mode, s.call_rs, rows_pad, s.call_a,
                                       s.call_sums, s.call_max, st);
        else if (s.call_sums)
            rc = rts_pp_rows_from_faces_staged(ctx, ctx->d_illum, N, N, (int)M, (int)kpad, nullptr, mode, s.call_rs,
                                               rows_pad, s.call_a, s.call_sums, s.call_max, st);
        else
            rc = rts_pp_rows_from_faces(ctx, ctx->d_illum, N, N, (int)M, (int)kpad, nullptr, mode, s.call_rs, rows_pad,
                                        s.call_a, st);
        if (rc == RTS_OK) rc = record_on(ctx, s.ev_prep, st);
        if (rc != RTS_OK) return rc;
        s.call_version = ctx->inputs_version;
        s.prep_slot = slot;
        for (bool& b : s.prep_served) b = false;
    }
    if ((rc = rts_group_step(s.slot[slot], 0, st)) != RTS_OK) return rc;
    if ((rc = record_on(ctx, s.ev_use[slot], st)) != RTS_OK) return rc;
    s.use_recorded[slot] = true;
    return RTS_OK;
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
                              p->fp16 ? p->rs + p->rows_pad : nullptr, p->mode, ctx->d_S, st);
    if (rc != RTS_OK) return rc;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(ibar_host, ctx->d_S, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

void rts_split_free(rts_ctx* ctx)
{
    rts_split_state& s = ctx->split;
    rts_group_batch_free(s.iter);
    for (int i = 0; i < RTS_STREAM_COUNT; ++i) rts_group_batch_free(s.slot[i]);
    free_call_rows(ctx);
    if (s.ev_prep) cudaEventDestroy(s.ev_prep);
    for (cudaEvent_t e : s.ev_use)
        if (e) cudaEventDestroy(e);
    if (s.ev_sent) cudaEventDestroy(s.ev_sent);
    if (s.ev_eager) cudaEventDestroy(s.ev_eager);
    if (s.eager_st) {
        cudaStreamSynchronize(s.eager_st);
        cudaStreamDestroy(s.eager_st);
    }
    for (int i = 0; i < RTS_HOST_CHUNKS; ++i) {
        rts_group_batch_free(s.chunk[i]);
        if (s.ev_in[i]) cudaEventDestroy(s.ev_in[i]);
        if (s.ev_done[i]) cudaEventDestroy(s.ev_done[i]);
    }
    if (s.ev_start) cudaEventDestroy(s.ev_start);
    if (s.copy_in) cudaStreamDestroy(s.copy_in);
    if (s.copy_out) cudaStreamDestroy(s.copy_out);
    s = rts_split_state();
}
