// rts_group.cu -- batched split-precision scattering integrals: many
// independent problems (own cell count, direction set, phase kernel,
// precision, groups, albedo) resident on the device, one persistent grouped
// tcgen05 launch per source-iteration step, optionally replayed from a CUDA
// graph.  The context's own source iteration (rts_solve_*) and host-buffer
// calls (rts_scattering_update) run on the same kernel through private
// one-problem batches (rts_split.cu).
//
// Reference counterpart: the reference solves one problem per process and
// launches d_GetS_MPI_Stream per call (cuda/cuda_solve.cu:89-111); batching,
// graphs and admission have no counterpart there.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "rts_group.h"
#include "rts_internal.h"
#include "rts_ptx.cuh"

namespace {
#include "rts_group_kernel.cuh"

int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn(rts_ctx* ctx)
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (fn) return fn;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
        cudaGetLastError();
        rts_fail(ctx, RTS_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        return nullptr;
    }
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return fn;
}

// 2-D map over interleaved split rows [rows][units] (16-bit units): box of
// box_cols halves x box_rows; the MMA operands use 64 x rows with a 128-byte
// swizzle, the relaxation 8 x 32 unswizzled (16 bytes of each of 32 rows).
int make_map(rts_ctx* ctx, void* map, const void* base, int64_t rows, int64_t units, int box_rows, int box_cols = 64,
             bool swizzle = true)
{
    auto enc = encode_fn(ctx);
    if (!enc) return RTS_ERR_CUDA;
    cuuint64_t dims[2] = {(cuuint64_t)units, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(units * 2)};
    cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1u, 1u};
    CUresult r = enc(reinterpret_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void*>(base),
                     dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return rts_fail(ctx, RTS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) for %lld x %lld", (int)r,
                        (long long)rows, (long long)units);
    return RTS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// problem and batch objects
// ---------------------------------------------------------------------------
struct rts_batch {
    rts_ctx* ctx = nullptr;
    std::vector<GProb*> probs;
    int64_t next_id = 1;
    GroupProblem* d_table = nullptr;
    size_t table_cap = 0;
    std::vector<GroupProblem> h_table;
    bool dirty = true;
    int table_relax = -1;
    int table_epoch = -1;  // ctx->tuning_epoch the table was built with
    unsigned long long* d_resid = nullptr;
    size_t resid_cap = 0;
    void* staging = nullptr;  // FP32 Ibar / FP64 W scratch for set-up
    size_t staging_bytes = 0;
    double* d_dirs = nullptr;  // xyz + area scratch
    size_t dirs_cap = 0;
    bool table_energy = false;  // a problem of the device table keeps the energy partial sums
    cudaGraphExec_t gexec = nullptr;
    int graph_steps = 0, graph_relax = 0;
    int64_t total_tiles = 0;
    int64_t steps = 0;
    GroupProblem* h_pin[2] = {nullptr, nullptr};  // pinned staging of subset tables
    size_t pin_cap = 0;
    cudaEvent_t pin_ev[2] = {nullptr, nullptr};
    int pin_next = 0;
};

namespace {

// frees are stream-ordered: after the work already queued on `st`
void free_prob(rts_ctx* ctx, GProb* p, cudaStream_t st)
{
    const size_t abytes = (size_t)(p->rows_pad * p->units * 2);
    rts_pfree(ctx, p->wc, (size_t)(p->mpad * p->units * 2), st);
    rts_pfree(ctx, p->cs, (size_t)(2 * p->mpad * 4), st);
    if (!p->a_ext) rts_pfree(ctx, p->a[0], abytes, st);
    rts_pfree(ctx, p->a[1], abytes, st);
    if (!p->a_ext) rts_pfree(ctx, p->rs, (size_t)(2 * p->rows_pad * 4), st);
    rts_pfree(ctx, p->B, (size_t)(p->rows * 4), st);
    rts_pfree(ctx, p->lam, (size_t)(p->groups * 4), st);
    rts_pfree(ctx, p->S32, (size_t)(p->rows * p->Mout * 4), st);
    rts_pfree(ctx, p->vrow, (size_t)((p->kpad + 4) * 4), st);
    rts_pfree(ctx, p->part, (size_t)(p->n_tiles * 4 * p->rows_pad * 16), st);
    rts_pfree(ctx, p->delta, (size_t)(p->rows_pad * 4), st);
    rts_pfree(ctx, p->ex, (size_t)(p->rows_pad * 8), st);
    delete p;
}

void free_prob(rts_ctx* ctx, GProb* p) { free_prob(ctx, p, ctx->streams[RTS_STREAM_SCATTERING_1]); }

void drop_graph(rts_batch* b)
{
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
    b->graph_steps = 0;
}

int ensure_scratch(rts_batch* b, size_t bytes, cudaStream_t st)
{
    if (b->staging_bytes >= bytes) return RTS_OK;
    rts_pfree(b->ctx, b->staging, b->staging_bytes, st);
    b->staging = nullptr;
    b->staging_bytes = 0;
    int rc = rts_pmalloc(b->ctx, &b->staging, bytes, "batch staging", st);
    if (rc == RTS_OK) b->staging_bytes = bytes;
    return rc;
}

}  // namespace

// Constant relative correction of the tensor core's truncating FP32
// accumulation, applied to every finished sum: none unless the caller sets
// one (RTS_TUNE_BIAS n > 0: n * 1e-10).  Each accumulate inside tcgen05.mma
// rounds toward zero, so sums come out low by ~1e-7 of themselves; how much
// depends on how the partial sums grow inside each MMA, i.e. on the data.
// Relaxed iterations, where the loss would compound, correct each cell from
// the conserved sum of its integrals instead (rts_group_kernel.cuh); a single
// evaluation keeps the loss of one pass.
float rts_group_bias(const rts_ctx* ctx, int, int)
{
    if (ctx->split_bias > 0) return (float)(ctx->split_bias * 1e-10);
    return 0.0f;
}

int64_t rts_group_energy_bytes(int64_t kpad, int64_t rows_pad, int n_tiles)
{
    return (kpad + 4) * 4 + (int64_t)n_tiles * 4 * rows_pad * 16 + rows_pad * 12;
}

// Tile geometry of a problem: out-direction tiles of at most G_BN (256), balanced.
void rts_group_geometry(int64_t Min, int64_t Mout, int64_t rows, int bn_override, int* bn, int* n_tiles,
                        int64_t* kpad, int64_t* mpad, int64_t* rows_pad, int64_t* m_tiles)
{
    int b = bn_override;
    if (b <= 0) {
        const int64_t nt = (Mout + G_BN - 1) / G_BN;
        b = (int)round_up((Mout + nt - 1) / nt, 16);
    }
    b = std::min(std::max(b, 16), G_BN);
    *bn = b;
    *n_tiles = (int)((Mout + b - 1) / b);
    *mpad = (int64_t)(*n_tiles) * b;
    *kpad = round_up(Min, 32);
    *rows_pad = round_up(rows, G_BM);
    *m_tiles = *rows_pad / G_BM;
}

int64_t rts_group_footprint(int64_t N, int64_t M, int64_t groups, bool iterative, int mode)
{
    int bn, nt;
    int64_t kpad, mpad, rows_pad, mt;
    const int64_t rows = N * groups;
    // an iteration's tiles also cover the correction's extra output column
    rts_group_geometry(M, iterative ? M + 1 : M, rows, 0, &bn, &nt, &kpad, &mpad, &rows_pad, &mt);
    const int64_t units = (mode == 2 ? 4 : 2) * kpad;
    int64_t bytes = mpad * units * 2 + 2 * mpad * 4 + 2 * rows_pad * 4 + rows * 4 + groups * 4;
    bytes += (iterative ? 2 : 1) * rows_pad * units * 2;
    if (iterative) bytes += rows * M * 4 + rts_group_energy_bytes(kpad, rows_pad, nt);
    return bytes;
}

// Creates a problem: allocations, W (phase kernel on the given directions)
// split into rows, tensor maps.  A rows, B and lambda are filled by the caller.
int rts_group_new_problem(rts_batch* b, int64_t N, int64_t Min, int64_t Mout, int64_t groups, const double* W_dev,
                          int ldw, int mode, int flush, int bn_override, bool iterative, GProb** out,
                          cudaStream_t st, uint16_t* ext_a, float* ext_rs)
{
    if ((ext_a != nullptr) != (ext_rs != nullptr) || (ext_a && (iterative || groups != 1)))
        return rts_fail(b->ctx, RTS_ERR_INVALID_ARGUMENT, "shared split rows need a single evaluation of one group");
    const bool fp16 = mode == 1;
    rts_ctx* ctx = b->ctx;
    GProb* p = new GProb();
    p->N = N;
    p->M = Min;
    p->Mout = Mout;
    p->groups = groups;
    p->rows = N * groups;
    p->fp16 = fp16;
    p->mode = mode;
    p->flush = std::min(std::max(flush, 1), G_MAX_FLUSH);
    {  // the autotuner's width (problems of all M out-directions without a width of their own) and tile order
        int tbn = 0, torder = 0;
        if (rts_tuned_tile(ctx, Min, mode, p->flush, p->rows, &tbn, &torder)) {
            if (bn_override <= 0 && Mout == Min) bn_override = tbn;
            p->order = torder;
        }
    }
    // the conservation correction of relaxed steps (iterations over all M
    // out-directions) takes one extra output column, index Mout: its W^T row
    // gives sum_j d_j (W^T x)_j (rts_pp_w_stats).  Every tiling has it.
    const bool energy = iterative && Mout == Min;
    rts_group_geometry(Min, energy ? Mout + 1 : Mout, p->rows, bn_override, &p->bn, &p->n_tiles, &p->kpad, &p->mpad,
                       &p->rows_pad, &p->m_tiles);
    int rc;
    void* q;
    if (!st) st = ctx->streams[RTS_STREAM_SCATTERING_1];
#define GP_ALLOC(field, nbytes, name)                                 \
    if ((rc = rts_pmalloc(ctx, &q, (nbytes), name, st)) != RTS_OK) { \
        free_prob(ctx, p, st);                                        \
        return rc;                                                    \
    }                                                                 \
    p->field = (decltype(p->field))q;                                 \
    p->bytes += (nbytes);
    p->units = (mode == 2 ? 4 : 2) * p->kpad;
    const size_t abytes = (size_t)(p->rows_pad * p->units * 2);
    GP_ALLOC(wc, (size_t)(p->mpad * p->units * 2), "split W");
    GP_ALLOC(cs, (size_t)(2 * p->mpad * 4), "W column scales");
    if (ext_a) {
        p->a_ext = true;
        p->a[0] = ext_a;
        p->rs = ext_rs;
    } else {
        GP_ALLOC(a[0], abytes, "split Ibar");
        GP_ALLOC(rs, (size_t)(2 * p->rows_pad * 4), "Ibar row scales");
    }
    if (iterative) {
        GP_ALLOC(a[1], abytes, "split Ibar (next)");
    }
    GP_ALLOC(B, (size_t)(p->rows * 4), "source B");
    GP_ALLOC(lam, (size_t)(p->groups * 4), "albedo");
    if (iterative) {
        GP_ALLOC(S32, (size_t)(p->rows * p->Mout * 4), "FP32 scattering");
    }
    if (energy) {
        GP_ALLOC(vrow, (size_t)((p->kpad + 4) * 4), "W row sums");
        GP_ALLOC(part, (size_t)(p->n_tiles * 4 * p->rows_pad * 16), "energy partial sums");
        GP_ALLOC(delta, (size_t)(p->rows_pad * 4), "energy corrections");
        GP_ALLOC(ex, (size_t)(p->rows_pad * 8), "conserved sums");
    }
#undef GP_ALLOC
    if (!ext_a) RTS_CUDA_TRY(ctx, cudaMemsetAsync(p->a[0], 0, abytes, st));
    if (p->a[1]) RTS_CUDA_TRY(ctx, cudaMemsetAsync(p->a[1], 0, abytes, st));
    if (p->S32) RTS_CUDA_TRY(ctx, cudaMemsetAsync(p->S32, 0, (size_t)(p->rows * p->Mout * 4), st));
    rc = rts_group_set_w(ctx, p, W_dev, ldw, st);
    if (rc == RTS_OK) rc = make_map(ctx, p->maps[2], p->wc, p->mpad, p->units, p->bn);
    if (rc == RTS_OK) rc = make_map(ctx, p->maps[0], p->a[0], p->rows_pad, p->units, G_BM);
    if (rc == RTS_OK && p->a[1]) rc = make_map(ctx, p->maps[1], p->a[1], p->rows_pad, p->units, G_BM);
    if (rc == RTS_OK) rc = make_map(ctx, p->rmaps[0], p->a[0], p->rows_pad, p->units, 32, 8, false);
    if (rc == RTS_OK && p->a[1]) rc = make_map(ctx, p->rmaps[1], p->a[1], p->rows_pad, p->units, 32, 8, false);
    if (rc != RTS_OK) {
        free_prob(ctx, p, st);
        return rc;
    }
    if (!p->a[1]) memcpy(p->maps[1], p->maps[0], 128);
    if (!p->a[1]) memcpy(p->rmaps[1], p->rmaps[0], 128);
    *out = p;
    return RTS_OK;
}

int rts_group_set_w(rts_ctx* ctx, GProb* p, const double* W_dev, int ldw, cudaStream_t st)
{
    const int Min = (int)p->M, Mout = (int)p->Mout;
    if (!p->vrow)
        return rts_pp_split_w(ctx, W_dev, Min, Mout, ldw, (int)p->kpad, (int)p->mpad, p->mode, p->wc, p->cs, st);
    // the correction's statistics and extra row (FP64 scratch, stream-ordered)
    void* scratch = nullptr;
    const size_t sbytes = (size_t)Min * 2 * sizeof(double);
    int rc = rts_pmalloc(ctx, &scratch, sbytes, "W statistics scratch", st);
    if (rc != RTS_OK) return rc;
    double* v64 = static_cast<double*>(scratch);
    double* u = v64 + Min;
    rc = rts_pp_w_stats(ctx, W_dev, Min, Mout, ldw, (int)p->kpad, p->vrow, v64, u, st);
    if (rc == RTS_OK)
        rc = rts_pp_split_w(ctx, W_dev, Min, Mout, ldw, (int)p->kpad, (int)p->mpad, p->mode, p->wc, p->cs, st, u);
    rts_pfree(ctx, scratch, sbytes, st);
    return rc;
}

int rts_group_reset_energy(rts_ctx* ctx, GProb* p, cudaStream_t st)
{
    if (!p->delta) return RTS_OK;
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(p->delta, 0, (size_t)(p->rows_pad * 4), st));
    group_energy_init_kernel<<<(unsigned)((p->rows * 32 + 255) / 256), 256, 0, st>>>(p->a[p->cur], p->rows, (int)p->kpad,
                                                                                  (int)p->M, p->mode, p->vrow, p->rs,
                                                                                  p->ex);
    RTS_CHECK_LAUNCH(ctx, "group_energy_init_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_group_attach(rts_batch* b, GProb* p, int64_t* id)
{
    p->id = b->next_id++;
    b->probs.push_back(p);
    b->dirty = true;
    drop_graph(b);
    if (id) *id = p->id;
    return RTS_OK;
}

GProb* rts_group_find(rts_batch* b, int64_t id, size_t* index)
{
    for (size_t i = 0; i < b->probs.size(); ++i)
        if (b->probs[i]->id == id) {
            if (index) *index = i;
            return b->probs[i];
        }
    return nullptr;
}

int rts_group_batch_new(rts_ctx* ctx, rts_batch** out)
{
    rts_batch* b = new rts_batch();
    b->ctx = ctx;
    *out = b;
    return RTS_OK;
}

void rts_group_batch_free(rts_batch* b)
{
    if (!b) return;
    rts_ctx* ctx = b->ctx;
    for (int i = 0; i < RTS_STREAM_COUNT; ++i) cudaStreamSynchronize(ctx->streams[i]);  // a batch may run on any slot
    drop_graph(b);
    for (GProb* p : b->probs) free_prob(ctx, p);
    rts_dfree(ctx, b->d_table, b->table_cap * sizeof(GroupProblem));
    rts_dfree(ctx, b->d_resid, b->resid_cap * sizeof(unsigned long long));
    rts_pfree(ctx, b->staging, b->staging_bytes, ctx->streams[RTS_STREAM_SCATTERING_1]);
    rts_pfree(ctx, b->d_dirs, b->dirs_cap * sizeof(double), ctx->streams[RTS_STREAM_SCATTERING_1]);
    for (int k = 0; k < 2; ++k) {
        if (b->h_pin[k]) cudaFreeHost(b->h_pin[k]);
        if (b->pin_ev[k]) cudaEventDestroy(b->pin_ev[k]);
    }
    delete b;
}

static bool relaxes(const GProb* p, int relax)
{
    return p->S32 != nullptr && relax && p->a[1] && p->Mout == p->M;
}

// One problem's entry of the device table: entry `i`, its tiles starting at
// `tiles` (advanced past them).
static void fill_entry(rts_batch* b, GProb* p, int relax, size_t i, int64_t& tiles, GroupProblem& g)
{
    rts_ctx* ctx = b->ctx;
    memset(&g, 0, sizeof(g));
    memcpy(&g.mapA[0], p->maps[0], 128);
    memcpy(&g.mapA[1], p->maps[1], 128);
    memcpy(&g.mapW, p->maps[2], 128);
    memcpy(&g.mapR[0], p->rmaps[0], 128);
    memcpy(&g.mapR[1], p->rmaps[1], 128);
    g.N = p->N;
    g.ldS = p->ldS > 0 ? p->ldS : p->N;
    g.rows = p->rows;
    g.tile_begin = tiles;
    g.m_tiles = (int)p->m_tiles;
    g.n_tiles = p->n_tiles;
    g.Mout = (int)p->Mout;
    g.kpad = (int)p->kpad;
    g.kblocks = (int)(p->kpad / (p->mode == 2 ? 16 : 32));
    g.bn = p->bn;
    g.flush = p->flush;
    g.order = p->order;
    g.groups = (int)p->groups;
    g.idesc = rts_ptx::idesc_split(p->mode, G_BM, p->bn);
    g.bias = rts_group_bias(ctx, p->mode, p->flush);
    g.fp16 = p->fp16 ? 1 : 0;
    g.tf32 = p->mode == 2 ? 1 : 0;
    // a quarter of the tile per epilogue column slice, so that narrow tiles keep every epilogue warp busy
    g.sw = std::min(64, (int)round_up((p->bn + 3) / 4, 16));
    g.cur = p->cur;
    g.relax = relaxes(p, relax) ? 1 : 0;
    g.flip = g.relax;
    g.tile_off = 0;
    g.residual = p->S32 != nullptr ? 1 : 0;
    g.rs = p->fp16 ? p->rs : nullptr;
    g.rs_inv = p->fp16 ? p->rs + p->rows_pad : nullptr;
    g.cs_inv = p->fp16 ? p->cs + p->mpad : nullptr;
    g.B = p->use_B ? p->B : nullptr;
    g.lam = p->lam;
    g.S32 = p->S32;
    g.S64 = p->S64;
    g.a[0] = p->a[0];
    g.a[1] = p->a[1] ? p->a[1] : p->a[0];
    g.resid = b->d_resid + i;
    // RTS_TUNE_BIAS -1 switches the conservation-based correction off; it
    // applies to relaxed steps (a step without relaxation leaves the input)
    const bool energy = p->part != nullptr && ctx->split_bias >= 0 && relaxes(p, relax);
    g.vrow = energy ? p->vrow : nullptr;
    g.part = energy ? reinterpret_cast<int4*>(p->part) : nullptr;
    g.delta = energy ? p->delta : nullptr;
    g.ex = energy ? p->ex : nullptr;
    g.rsb = p->rs;
    p->slot = (int)i;
    tiles += p->m_tiles * p->n_tiles;
}

// Device table and residual slots for at least n problems.
static int ensure_table(rts_batch* b, size_t n, cudaStream_t st)
{
    rts_ctx* ctx = b->ctx;
    if (n <= b->table_cap) return RTS_OK;
    cudaStreamSynchronize(st);
    rts_dfree(ctx, b->d_table, b->table_cap * sizeof(GroupProblem));
    rts_dfree(ctx, b->d_resid, b->resid_cap * sizeof(unsigned long long));
    b->d_table = nullptr;
    b->d_resid = nullptr;
    b->table_cap = b->resid_cap = 0;
    const size_t cap = std::max<size_t>(16, n * 2);
    void* q;
    int rc = rts_dmalloc(ctx, &q, cap * sizeof(GroupProblem), "batch table");
    if (rc != RTS_OK) return rc;
    b->d_table = (GroupProblem*)q;
    rc = rts_dmalloc(ctx, &q, cap * sizeof(unsigned long long), "batch residuals");
    if (rc != RTS_OK) return rc;
    b->d_resid = (unsigned long long*)q;
    b->table_cap = b->resid_cap = cap;
    return RTS_OK;
}

// Build the device table for the next launch(es).
static int upload_table(rts_batch* b, int relax, cudaStream_t st)
{
    rts_ctx* ctx = b->ctx;
    if (!b->dirty && b->table_relax == relax && b->table_epoch == ctx->tuning_epoch) return RTS_OK;
    const size_t n = b->probs.size();
    int rc = ensure_table(b, n, st);
    if (rc != RTS_OK) return rc;
    b->h_table.assign(n, GroupProblem());
    int64_t tiles = 0;
    b->table_energy = false;
    for (size_t i = 0; i < n; ++i) {
        fill_entry(b, b->probs[i], relax, i, tiles, b->h_table[i]);
        b->table_energy |= b->h_table[i].part != nullptr;
    }
    // the energy instantiation runs relaxed iterations only (no FP64 outputs)
    for (size_t i = 0; i < n; ++i) b->table_energy &= b->h_table[i].S64 == nullptr;
    b->total_tiles = tiles;
    if (n) RTS_CUDA_TRY(ctx, cudaMemcpyAsync(b->d_table, b->h_table.data(), n * sizeof(GroupProblem),
                                             cudaMemcpyHostToDevice, st));
    // the pageable source must outlive the copy
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    b->dirty = false;
    b->table_relax = relax;
    b->table_epoch = ctx->tuning_epoch;
    return RTS_OK;
}

// Dynamic shared memory of both instantiations of the kernel.
static cudaError_t set_kernel_smem()
{
    cudaError_t e = cudaFuncSetAttribute(group_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G_SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(group_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G_SMEM);
    return e;
}

int rts_group_prepare(rts_batch* b, int relax, cudaStream_t st)
{
    rts_ctx* ctx = b->ctx;
    if (b->probs.empty()) return RTS_OK;
    RTS_CUDA_TRY(ctx, set_kernel_smem());
    return upload_table(b, relax, st);
}

static int enqueue_step(rts_batch* b, int relax, cudaStream_t st, int n)
{
    rts_ctx* ctx = b->ctx;
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(b->d_resid, 0, n * sizeof(unsigned long long), st));
    const int64_t grid = std::min<int64_t>((int64_t)ctx->num_sms * G_CTAS_PER_SM, b->total_tiles);
    if (grid > 0) {
        rts_timing_begin(ctx, st);
        // the energy bookkeeping is compiled in only where a relaxed problem of the launch uses it
        if (relax && b->table_energy)
            group_kernel<true><<<(unsigned)grid, G_THREADS, G_SMEM, st>>>(b->d_table, n, b->total_tiles, ctx->d_flag);
        else
            group_kernel<false><<<(unsigned)grid, G_THREADS, G_SMEM, st>>>(b->d_table, n, b->total_tiles, ctx->d_flag);
        rts_timing_end(ctx, st);
        RTS_CHECK_LAUNCH(ctx, "group_kernel");
        ctx->launches++;
    }
    if (relax) {
        // each cell's correction of the next step, after a launch that kept
        // the partial sums (problems without the buffers return at once);
        // then the buffer flip
        if (b->table_energy) {
            const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(2 * ctx->num_sms, 1 << 12));
            group_energy_kernel<<<dim3(gx, (unsigned)n), 256, 0, st>>>(b->d_table, n);
            RTS_CHECK_LAUNCH(ctx, "group_energy_kernel");
            ctx->launches++;
        }
        group_flip_kernel<<<(n + 127) / 128, 128, 0, st>>>(b->d_table, n);
        RTS_CHECK_LAUNCH(ctx, "group_flip_kernel");
        ctx->launches++;
    }
    return RTS_OK;
}

static void host_flip(rts_batch* b, int relax, int times)
{
    if (!relax || !(times & 1)) return;
    for (size_t i = 0; i < b->probs.size(); ++i) {
        GProb* p = b->probs[i];
        if (p->S32 && p->a[1]) {
            p->cur ^= 1;
            b->h_table[i].cur ^= 1;  // the device table was flipped in place
        }
    }
}

int rts_group_step(rts_batch* b, int relax, cudaStream_t st)
{
    rts_ctx* ctx = b->ctx;
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED,
                "the tensor-core path needs a Blackwell (sm_10x) device, found sm_%d%d", ctx->cc_major, ctx->cc_minor);
    if (b->probs.empty()) return RTS_OK;
    RTS_CUDA_TRY(ctx, set_kernel_smem());
    int rc = upload_table(b, relax, st);
    if (rc != RTS_OK) return rc;
    rc = enqueue_step(b, relax, st, (int)b->probs.size());
    if (rc != RTS_OK) return rc;
    host_flip(b, relax, 1);
    b->steps++;
    return RTS_OK;
}

// Part of a step of some of the batch's problems (the others keep their
// state): problem ids[i] runs tiles [first[i], first[i] + count[i]) of its
// current step, and its step ends in this launch when that range reaches its
// last tile (then, relaxing, its Ibar buffers flip).  The table is rebuilt
// for these pieces in a pinned host buffer (two, used in turn) and copied
// without a host synchronisation.  Residuals are those of this launch's tiles.
int rts_group_step_pieces(rts_batch* b, int relax, const int64_t* ids, const int64_t* first, const int64_t* count,
                          int n, cudaStream_t st)
{
    rts_ctx* ctx = b->ctx;
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED, "the tensor-core path needs a Blackwell device");
    if (n <= 0) return RTS_OK;
    std::vector<GProb*> sel((size_t)n);
    for (int i = 0; i < n; ++i) {
        sel[i] = rts_group_find(b, ids[i], nullptr);
        RTS_REQUIRE(ctx, sel[i], RTS_ERR_INVALID_ARGUMENT, "no problem with id %lld in the batch", (long long)ids[i]);
        const int64_t tiles = sel[i]->m_tiles * sel[i]->n_tiles;
        const int64_t f = first ? first[i] : 0, c = count ? count[i] : tiles;
        RTS_REQUIRE(ctx, f >= 0 && c > 0 && f + c <= tiles, RTS_ERR_INVALID_ARGUMENT,
                    "tiles [%lld,%lld) outside the problem's %lld", (long long)f, (long long)(f + c), (long long)tiles);
    }
    RTS_CUDA_TRY(ctx, set_kernel_smem());
    int rc = ensure_table(b, (size_t)n, st);
    if (rc != RTS_OK) return rc;
    if (b->pin_cap < (size_t)n) {
        for (int k = 0; k < 2; ++k) {
            if (b->pin_ev[k]) cudaEventSynchronize(b->pin_ev[k]);
            if (b->h_pin[k]) cudaFreeHost(b->h_pin[k]);
            b->h_pin[k] = nullptr;
        }
        b->pin_cap = 0;
        const size_t cap = std::max<size_t>(16, (size_t)n * 2);
        for (int k = 0; k < 2; ++k) {
            RTS_CUDA_TRY(ctx, cudaMallocHost(&b->h_pin[k], cap * sizeof(GroupProblem)));
            if (!b->pin_ev[k]) RTS_CUDA_TRY(ctx, cudaEventCreateWithFlags(&b->pin_ev[k], cudaEventDisableTiming));
        }
        b->pin_cap = cap;
    }
    const int k = b->pin_next;
    b->pin_next ^= 1;
    RTS_CUDA_TRY(ctx, cudaEventSynchronize(b->pin_ev[k]));  // its previous copy has been consumed
    int64_t total = 0;
    b->table_energy = false;
    bool energy_blocked = false;
    for (int i = 0; i < n; ++i) {
        GroupProblem& g = b->h_pin[k][i];
        int64_t ignored = 0;
        fill_entry(b, sel[i], relax, (size_t)i, ignored, g);
        b->table_energy |= g.part != nullptr;
        if (g.S64) energy_blocked = true;
        const int64_t tiles = sel[i]->m_tiles * sel[i]->n_tiles;
        const int64_t f = first ? first[i] : 0, c = count ? count[i] : tiles;
        g.tile_begin = total;
        g.tile_off = f;
        g.flip = (g.relax && f + c == tiles) ? 1 : 0;
        total += c;
    }
    if (energy_blocked) b->table_energy = false;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(b->d_table, b->h_pin[k], (size_t)n * sizeof(GroupProblem),
                                      cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaEventRecord(b->pin_ev[k], st));
    b->total_tiles = total;
    b->dirty = true;  // the device table no longer holds the whole batch
    rc = enqueue_step(b, relax, st, n);
    if (rc != RTS_OK) return rc;
    for (int i = 0; i < n; ++i) {
        const int64_t tiles = sel[i]->m_tiles * sel[i]->n_tiles;
        const int64_t f = first ? first[i] : 0, c = count ? count[i] : tiles;
        if (relaxes(sel[i], relax) && f + c == tiles) sel[i]->cur ^= 1;
    }
    b->steps++;
    return RTS_OK;
}

int rts_group_step_subset(rts_batch* b, int relax, const int64_t* ids, int n, cudaStream_t st)
{
    return rts_group_step_pieces(b, relax, ids, nullptr, nullptr, n, st);
}

int64_t rts_group_problem_tiles(rts_batch* b, int64_t id)
{
    GProb* p = rts_group_find(b, id, nullptr);
    return p ? p->m_tiles * p->n_tiles : 0;
}

int rts_group_capture(rts_batch* b, int steps, int relax)
{
    rts_ctx* ctx = b->ctx;
    RTS_REQUIRE(ctx, steps > 0 && steps <= 4096, RTS_ERR_INVALID_ARGUMENT, "graph steps %d outside [1,4096]", steps);
    RTS_REQUIRE(ctx, !b->probs.empty(), RTS_ERR_BAD_STATE, "capture of an empty batch");
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED, "the tensor-core path needs a Blackwell device");
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, set_kernel_smem());
    int rc = upload_table(b, relax, st);
    if (rc != RTS_OK) return rc;
    drop_graph(b);
    const bool was_timing = ctx->timing;
    ctx->timing = false;  // no event records inside the graph
    RTS_CUDA_TRY(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int64_t launches0 = ctx->launches;
    for (int s = 0; s < steps && rc == RTS_OK; ++s) rc = enqueue_step(b, relax, st, (int)b->probs.size());
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    ctx->timing = was_timing;
    ctx->launches = launches0;  // counted when the graph is replayed
    if (rc != RTS_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return rts_fail(ctx, RTS_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        b->gexec = nullptr;
        return rts_fail(ctx, RTS_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
    }
    b->graph_steps = steps;
    b->graph_relax = relax;
    return RTS_OK;
}

int rts_group_replay(rts_batch* b)
{
    rts_ctx* ctx = b->ctx;
    RTS_REQUIRE(ctx, b->gexec && !b->dirty, RTS_ERR_BAD_STATE,
                "no captured graph (or the batch changed since the capture)");
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    rts_timing_begin(ctx, st);
    RTS_CUDA_TRY(ctx, cudaGraphLaunch(b->gexec, st));
    rts_timing_end(ctx, st);
    ctx->launches += (int64_t)b->graph_steps * (b->graph_relax ? 2 : 1);
    host_flip(b, b->graph_relax, b->graph_steps);
    b->steps += b->graph_steps;
    return RTS_OK;
}

int64_t rts_group_total_tiles(rts_batch* b)
{
    int64_t tiles = 0;
    for (GProb* p : b->probs) tiles += p->m_tiles * p->n_tiles;
    return tiles;
}
rts_ctx* rts_group_ctx(rts_batch* b) { return b->ctx; }
size_t rts_group_count(rts_batch* b) { return b->probs.size(); }
unsigned long long* rts_group_resid_slot(rts_batch* b, size_t index) { return b->d_resid + index; }
int rts_group_scratch(rts_batch* b, size_t bytes, void** p, cudaStream_t st)
{
    int rc = ensure_scratch(b, bytes, st ? st : b->ctx->streams[RTS_STREAM_SCATTERING_1]);
    if (rc == RTS_OK) *p = b->staging;
    return rc;
}

int rts_group_dirs(rts_batch* b, const double* xyz, const double* area, int64_t M, double** d_xyz, double** d_area,
                   cudaStream_t st)
{
    rts_ctx* ctx = b->ctx;
    if (!st) st = ctx->streams[RTS_STREAM_SCATTERING_1];
    const size_t need = (size_t)(4 * M);
    if (b->dirs_cap < need) {
        rts_pfree(ctx, b->d_dirs, b->dirs_cap * sizeof(double), st);
        b->d_dirs = nullptr;
        b->dirs_cap = 0;
        void* q;
        int rc = rts_pmalloc(ctx, &q, need * sizeof(double), "batch directions", st);
        if (rc != RTS_OK) return rc;
        b->d_dirs = (double*)q;
        b->dirs_cap = need;
    }
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(b->d_dirs, xyz, (size_t)(3 * M) * 8, cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(b->d_dirs + 3 * M, area, (size_t)M * 8, cudaMemcpyHostToDevice, st));
    *d_xyz = b->d_dirs;
    *d_area = b->d_dirs + 3 * M;
    return RTS_OK;
}

int rts_group_remove(rts_batch* b, int64_t id) { return rts_group_remove_on(b, id, nullptr); }

// The problem's buffers are freed in the order of `st` (the scattering stream
// when null): after every launch or copy already queued there.
int rts_group_remove_on(rts_batch* b, int64_t id, cudaStream_t st)
{
    size_t idx = 0;
    GProb* p = rts_group_find(b, id, &idx);
    RTS_REQUIRE(b->ctx, p, RTS_ERR_INVALID_ARGUMENT, "no problem with id %lld in the batch", (long long)id);
    free_prob(b->ctx, p, st ? st : b->ctx->streams[RTS_STREAM_SCATTERING_1]);
    b->probs.erase(b->probs.begin() + (long)idx);
    b->dirty = true;
    drop_graph(b);
    return RTS_OK;
}

void rts_group_invalidate(rts_batch* b)
{
    if (!b) return;
    b->dirty = true;
    drop_graph(b);
}
