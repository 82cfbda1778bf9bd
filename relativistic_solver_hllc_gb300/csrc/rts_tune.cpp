// rts_tune.cpp -- autotuner of the grouped tensor-core kernel's schedule.
//
// A schedule is a drain period (K-slices accumulated on the tensor core per
// FP32 drain), a tile width (out-directions per tile) and a tile order.
// rts_autotune_schedule times every combination allowed for a direction
// count M and a precision on a synthetic Thomson problem of a given cell
// count:
//   * drain period: those the accuracy rule allows (rts_auto_flush: FP16 and
//     BF16 one K-slice, or one and two for smooth kernels; TF32 two);
//   * tile width: every distinct tiling of the out-directions (n tiles of
//     bn = 16 ceil(M / (16 n)) directions, bn from 64 to 256);
//   * tile order: the column tiles of a row tile in turn (a 128-row slab of
//     the split Ibar is read from DRAM once while its column tiles run side
//     by side on neighbouring SMs), or the row tiles of a column tile in turn.
// The fastest width and order of each drain period go into the context's
// table, keyed by (M, precision, drain period, cell bucket).  A problem then
// takes -- unless its caller fixes them -- the drain period with the shorter
// tuned time among those its own kernel allows (rts_tuned_flush), and that
// period's width and order (rts_tuned_tile), from the entry of the nearest
// cell bucket.  Width and order do not change any output's arithmetic (each
// output is summed over the same K-slices in the same order), so they give
// bit-identical results; the drain period changes the rounding, within the
// accuracy the rule guarantees.  rts_autotune is the width-only search at one
// drain period.  The table is saved to and loaded from a text file.
//
// No counterpart in the reference (its launch shape is fixed, cuda/cuda_solve.cu:94-99).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rts_group.h"
#include "rts_internal.h"

namespace {

int mode_precision(int mode)
{
    return mode == 1 ? RTS_PREC_FP16X3 : mode == 2 ? RTS_PREC_TF32X3 : RTS_PREC_BF16X3;
}

bool tensor_precision(int p)
{
    return p == RTS_PREC_FP16X3 || p == RTS_PREC_BF16X3 || p == RTS_PREC_TF32X3;
}

rts_tune_entry* find_entry(rts_ctx* ctx, int64_t M, int precision, int flush, int bucket)
{
    for (rts_tune_entry& e : ctx->tune)
        if (e.M == M && e.precision == precision && e.flush == flush && e.bucket == bucket) return &e;
    return nullptr;
}

void put_entry(rts_ctx* ctx, const rts_tune_entry& v)
{
    rts_tune_entry* e = find_entry(ctx, v.M, v.precision, v.flush, v.bucket);
    if (!e) {
        ctx->tune.push_back(v);
        return;
    }
    *e = v;
}

// Distance of an entry's cell bucket from a problem's (an entry without a
// bucket fits every problem, after an exact match).
double bucket_distance(const rts_tune_entry& e, int bucket)
{
    return e.bucket < 0 ? 0.5 : std::fabs((double)(e.bucket - bucket));
}

const rts_tune_entry* match(const rts_ctx* ctx, int64_t M, int precision, int flush, int bucket)
{
    const rts_tune_entry* best = nullptr;
    double bd = 1e300;
    for (const rts_tune_entry& e : ctx->tune) {
        if (e.M != M || e.precision != precision || e.flush != flush) continue;
        const double d = bucket_distance(e, bucket);
        if (d < bd) {
            bd = d;
            best = &e;
        }
    }
    return best;
}

// The automatic drain period of the tuning problem (Thomson, Fibonacci directions).
int auto_period(int64_t M, int precision)
{
    std::vector<double> xyz(3 * (size_t)M), area((size_t)M);
    double fa = 0.0;
    rts_synth_directions(M, xyz.data(), area.data(), &fa);
    return rts_auto_flush(xyz.data(), area.data(), M, fa, 0, M, RTS_PHASE_THOMSON, 0.0, precision);
}

// The distinct tilings of M out-directions.
std::vector<int> widths(int64_t M)
{
    std::vector<int> cand;
    for (int64_t nt = (M + 255) / 256; nt <= (M + 63) / 64; ++nt) {
        const int bn = (int)(((M + nt - 1) / nt + 15) / 16 * 16);
        if (bn > 256 || bn < 16) continue;
        if (std::find(cand.begin(), cand.end(), bn) == cand.end()) cand.push_back(bn);
        if (cand.size() >= 8) break;
    }
    if (cand.empty()) cand.push_back((int)std::min<int64_t>(256, (M + 15) / 16 * 16));
    return cand;
}

// One schedule on the synthetic problem: two warm-up steps, then the mean of
// five relaxed steps (CUDA events on the scattering stream).
int time_schedule(rts_ctx* ctx, int64_t M, int precision, int flush, int bn, int order, int64_t cells,
                  cudaEvent_t e0, cudaEvent_t e1, double* ms)
{
    rts_batch* b = nullptr;
    int rc = rts_batch_create(ctx, &b);
    if (rc != RTS_OK) return rc;
    rts_problem_desc d;
    memset(&d, 0, sizeof(d));
    d.N = cells;
    d.M = M;
    d.groups = 1;
    d.phase = RTS_PHASE_THOMSON;
    d.precision = precision;
    d.flush = flush;
    d.bn = bn;
    const double lam = 0.5;
    int64_t id = 0;
    rc = rts_batch_add_synthetic(b, &d, 17, 0.0, 1.0, 0.1, 1.0, &lam, &id);
    if (rc == RTS_OK) {
        GProb* p = rts_group_find(b, id, nullptr);
        if (p && p->order != order) {
            p->order = order;
            rts_group_invalidate(b);
        }
    }
    for (int w = 0; w < 2 && rc == RTS_OK; ++w) rc = rts_batch_step(b, 1);
    float t = 0.0f;
    const int reps = 5;
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    if (rc == RTS_OK) {
        cudaEventRecord(e0, st);
        for (int r = 0; r < reps && rc == RTS_OK; ++r) rc = rts_batch_step(b, 1);
        cudaEventRecord(e1, st);
        if (rc == RTS_OK) rc = rts_batch_sync(b, 10000000);
        if (rc == RTS_OK) cudaEventElapsedTime(&t, e0, e1);
    }
    rts_batch_destroy(b);
    *ms = (double)t / reps;
    return rc;
}

int64_t default_cells(const rts_ctx* ctx) { return (int64_t)ctx->num_sms * 128 * 4; }  // four waves of row tiles

}  // namespace

int rts_cells_bucket(const rts_ctx* ctx, int64_t rows)
{
    const double waves = (double)rows / ((double)std::max(ctx->num_sms, 1) * 128.0);
    return waves < 1.0 ? 0 : waves < 4.0 ? 1 : waves < 16.0 ? 2 : 3;
}

int rts_tuned_flush(const rts_ctx* ctx, int64_t M, int precision, int64_t rows, int cap)
{
    if (ctx->tune.empty() || cap <= 1 || precision == RTS_PREC_TF32X3) return cap;
    const int bucket = rts_cells_bucket(ctx, rows);
    const rts_tune_entry* top = match(ctx, M, precision, cap, bucket);
    if (!top) return cap;  // no evidence that a shorter period is faster
    int best = cap;
    double best_ms = top->ms;
    for (int f = 1; f < cap; ++f) {
        const rts_tune_entry* e = match(ctx, M, precision, f, bucket);
        if (e && bucket_distance(*e, bucket) == bucket_distance(*top, bucket) && e->ms < best_ms) {
            best = f;
            best_ms = e->ms;
        }
    }
    return best;
}

bool rts_tuned_tile(const rts_ctx* ctx, int64_t M, int mode, int flush, int64_t rows, int* bn, int* order)
{
    const rts_tune_entry* e = match(ctx, M, mode_precision(mode), std::max(flush, 1), rts_cells_bucket(ctx, rows));
    if (!e) return false;
    *bn = e->bn;
    *order = e->order;
    return true;
}

extern "C" int rts_autotune(rts_ctx* ctx, int64_t M, int precision, int flush, int64_t cells, int* best_bn,
                            double* best_ms, int* tried_bn, double* tried_ms, int capacity, int* tried)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, M >= 1 && M <= 65536, RTS_ERR_INVALID_ARGUMENT, "rts_autotune: M=%lld out of range",
                (long long)M);
    RTS_REQUIRE(ctx, tensor_precision(precision), RTS_ERR_INVALID_ARGUMENT,
                "rts_autotune: precision %d is not a tensor-core precision", precision);
    RTS_REQUIRE(ctx, flush >= 0 && flush <= 2, RTS_ERR_INVALID_ARGUMENT, "rts_autotune: flush %d outside [0,2]", flush);
    if (cells <= 0) cells = default_cells(ctx);
    RTS_REQUIRE(ctx, cells <= ((int64_t)1 << 26), RTS_ERR_INVALID_ARGUMENT, "rts_autotune: %lld cells",
                (long long)cells);
    if (flush == 0) flush = auto_period(M, precision);

    cudaEvent_t e0, e1;
    RTS_CUDA_TRY(ctx, cudaEventCreate(&e0));
    RTS_CUDA_TRY(ctx, cudaEventCreate(&e1));
    int best = 0, n_tried = 0, rc = RTS_OK;
    double best_t = 1e300;
    for (int bn : widths(M)) {
        double t = 0.0;
        if ((rc = time_schedule(ctx, M, precision, flush, bn, 0, cells, e0, e1, &t)) != RTS_OK) break;
        if (tried_bn && tried_ms && n_tried < capacity) {
            tried_bn[n_tried] = bn;
            tried_ms[n_tried] = t;
        }
        ++n_tried;
        if (t < best_t) {
            best_t = t;
            best = bn;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != RTS_OK) return rc;
    if (tried) *tried = n_tried;
    if (best_bn) *best_bn = best;
    if (best_ms) *best_ms = best_t;
    rts_tune_entry v;
    v.M = M;
    v.precision = precision;
    v.flush = flush;
    v.bucket = rts_cells_bucket(ctx, cells);
    v.bn = best;
    v.order = 0;
    v.ms = best_t;
    put_entry(ctx, v);
    ctx->tuning_epoch++;
    return RTS_OK;
}

extern "C" int rts_autotune_schedule(rts_ctx* ctx, int64_t M, int precision, int64_t cells, rts_tune_choice* best,
                                     rts_tune_choice* tried, int capacity, int* n_tried)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, M >= 1 && M <= 65536, RTS_ERR_INVALID_ARGUMENT, "rts_autotune_schedule: M=%lld out of range",
                (long long)M);
    RTS_REQUIRE(ctx, tensor_precision(precision), RTS_ERR_INVALID_ARGUMENT,
                "rts_autotune_schedule: precision %d is not a tensor-core precision", precision);
    RTS_REQUIRE(ctx, capacity >= 0 && (capacity == 0 || tried), RTS_ERR_INVALID_ARGUMENT,
                "rts_autotune_schedule: %d result slots without an array", capacity);
    if (cells <= 0) cells = default_cells(ctx);
    RTS_REQUIRE(ctx, cells <= ((int64_t)1 << 26), RTS_ERR_INVALID_ARGUMENT, "rts_autotune_schedule: %lld cells",
                (long long)cells);
    const int cap = auto_period(M, precision);
    const int bucket = rts_cells_bucket(ctx, cells);
    const int m_tiles = (int)((cells + 127) / 128);
    std::vector<int> periods;
    if (precision == RTS_PREC_TF32X3)
        periods.push_back(cap);
    else
        for (int f = 1; f <= cap; ++f) periods.push_back(f);

    cudaEvent_t e0, e1;
    RTS_CUDA_TRY(ctx, cudaEventCreate(&e0));
    RTS_CUDA_TRY(ctx, cudaEventCreate(&e1));
    int rc = RTS_OK, n = 0;
    rts_tune_choice overall;
    memset(&overall, 0, sizeof(overall));
    overall.ms = 1e300;
    std::vector<rts_tune_entry> found;
    for (int f : periods) {
        rts_tune_entry bf;
        bf.M = M;
        bf.precision = precision;
        bf.flush = f;
        bf.bucket = bucket;
        bf.ms = 1e300;
        for (int bn : widths(M)) {
            const int n_tiles = (int)((M + bn - 1) / bn);
            for (int order = 0; order < 2 && rc == RTS_OK; ++order) {
                if (order == 1 && (n_tiles == 1 || m_tiles == 1)) break;  // one order only
                double t = 0.0;
                if ((rc = time_schedule(ctx, M, precision, f, bn, order, cells, e0, e1, &t)) != RTS_OK) break;
                rts_tune_choice c;
                c.M = M;
                c.precision = precision;
                c.flush = f;
                c.bn = bn;
                c.order = order;
                c.bucket = bucket;
                c.ms = t;
                if (n < capacity) tried[n] = c;
                ++n;
                if (t < bf.ms) {
                    bf.ms = t;
                    bf.bn = bn;
                    bf.order = order;
                }
                if (t < overall.ms) overall = c;
            }
            if (rc != RTS_OK) break;
        }
        if (rc != RTS_OK) break;
        found.push_back(bf);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != RTS_OK) return rc;
    for (const rts_tune_entry& e : found) put_entry(ctx, e);
    ctx->tuning_epoch++;
    if (best) *best = overall;
    if (n_tried) *n_tried = n;
    return RTS_OK;
}

extern "C" int rts_autotune_save(rts_ctx* ctx, const char* path)
{
    if (!ctx || !path) return RTS_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "w");
    RTS_REQUIRE(ctx, f, RTS_ERR_INVALID_ARGUMENT, "cannot write %s", path);
    std::fprintf(f, "# rts schedule table: M precision flush cell_bucket bn order ms\n");
    for (const rts_tune_entry& e : ctx->tune)
        std::fprintf(f, "%lld %d %d %d %d %d %.9g\n", (long long)e.M, e.precision, e.flush, e.bucket, e.bn, e.order,
                     e.ms);
    const bool ok = std::fclose(f) == 0;
    RTS_REQUIRE(ctx, ok, RTS_ERR_INVALID_ARGUMENT, "error writing %s", path);
    return RTS_OK;
}

// Reads tables in this format and in the width-only one ("M precision flush
// bn ms": every cell bucket, first tile order).
extern "C" int rts_autotune_load(rts_ctx* ctx, const char* path)
{
    if (!ctx || !path) return RTS_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "r");
    RTS_REQUIRE(ctx, f, RTS_ERR_INVALID_ARGUMENT, "cannot read %s", path);
    char line[256];
    int rc = RTS_OK;
    std::vector<rts_tune_entry> read;
    while (std::fgets(line, sizeof(line), f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        long long M = 0;
        int prec = 0, fl = 0, bucket = -1, bn = 0, order = 0;
        double ms = 0.0;
        const int k = std::sscanf(line, "%lld %d %d %d %d %d %lf", &M, &prec, &fl, &bucket, &bn, &order, &ms);
        if (k != 7) {
            bucket = -1;
            order = 0;
            if (std::sscanf(line, "%lld %d %d %d %lf", &M, &prec, &fl, &bn, &ms) != 5) M = 0;
        }
        if (M < 1 || !tensor_precision(prec) || fl < 1 || fl > 2 || bucket < -1 || bucket > 3 || bn < 16 ||
            bn > 256 || bn % 16 != 0 || order < 0 || order > 1) {
            rc = rts_fail(ctx, RTS_ERR_INVALID_ARGUMENT, "%s: malformed entry: %s", path, line);
            break;
        }
        rts_tune_entry e;
        e.M = M;
        e.precision = prec;
        e.flush = fl;
        e.bucket = bucket;
        e.bn = bn;
        e.order = order;
        e.ms = ms;
        read.push_back(e);
    }
    std::fclose(f);
    if (rc != RTS_OK) return rc;
    for (const rts_tune_entry& e : read) put_entry(ctx, e);
    ctx->tuning_epoch++;
    return RTS_OK;
}
