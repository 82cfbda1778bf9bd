// rts_tune.cpp -- autotuner of the grouped tensor-core kernel's tile width.
//
// For a direction count M, precision and flush period, every distinct tiling
// of the out-directions (n tiles of bn = 16 * ceil(M / (16 n)) directions,
// bn from 64 to 256) is timed on a synthetic problem large enough to fill the
// GPU; the fastest bn is kept in the context's table and used for problems
// created with bn = 0 (rts_batch_add*, the context's own source iteration and
// host-buffer calls).  The table can be saved to and loaded from a text file
// (one line per entry: "M precision flush bn ms").  The tiling does not change
// any output's arithmetic (each output is summed over the same K-slices in the
// same order), so every bn gives bit-identical results.
//
// No counterpart in the reference (its launch shape is fixed, cuda/cuda_solve.cu:94-99).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rts_group.h"
#include "rts_internal.h"

namespace {

rts_tune_entry* find_entry(rts_ctx* ctx, int64_t M, int precision, int flush)
{
    for (rts_tune_entry& e : ctx->tune)
        if (e.M == M && e.precision == precision && e.flush == flush) return &e;
    return nullptr;
}

}  // namespace

int rts_tuned_bn(const rts_ctx* ctx, int64_t M, int mode, int flush)
{
    const int prec = mode == 1 ? RTS_PREC_FP16X3 : mode == 2 ? RTS_PREC_TF32X3 : RTS_PREC_BF16X3;
    const int fl = std::max(flush, 1);
    for (const rts_tune_entry& e : ctx->tune)
        if (e.M == M && e.precision == prec && std::max(e.flush, 1) == fl) return e.bn;
    return 0;
}

extern "C" int rts_autotune(rts_ctx* ctx, int64_t M, int precision, int flush, int64_t cells, int* best_bn,
                            double* best_ms, int* tried_bn, double* tried_ms, int capacity, int* tried)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, M >= 1 && M <= 65536, RTS_ERR_INVALID_ARGUMENT, "rts_autotune: M=%lld out of range",
                (long long)M);
    RTS_REQUIRE(ctx, precision == RTS_PREC_FP16X3 || precision == RTS_PREC_BF16X3 || precision == RTS_PREC_TF32X3,
                RTS_ERR_INVALID_ARGUMENT,
                "rts_autotune: precision %d is not a tensor-core precision", precision);
    RTS_REQUIRE(ctx, flush >= 0 && flush <= 2, RTS_ERR_INVALID_ARGUMENT, "rts_autotune: flush %d outside [0,2]", flush);
    if (cells <= 0) cells = (int64_t)ctx->num_sms * 128 * 4;  // four waves of row tiles
    if (flush == 0) {  // the automatic drain period of the tuning problem (Thomson, Fibonacci directions)
        std::vector<double> xyz(3 * (size_t)M), area((size_t)M);
        double fa = 0.0;
        rts_synth_directions(M, xyz.data(), area.data(), &fa);
        flush = rts_auto_flush(xyz.data(), area.data(), M, fa, 0, M, RTS_PHASE_THOMSON, 0.0, precision);
    }
    RTS_REQUIRE(ctx, cells <= ((int64_t)1 << 26), RTS_ERR_INVALID_ARGUMENT, "rts_autotune: %lld cells",
                (long long)cells);

    // the distinct tilings
    std::vector<int> cand;
    for (int64_t nt = (M + 255) / 256; nt <= (M + 63) / 64; ++nt) {
        const int bn = (int)(((M + nt - 1) / nt + 15) / 16 * 16);
        if (bn > 256 || bn < 16) continue;
        if (std::find(cand.begin(), cand.end(), bn) == cand.end()) cand.push_back(bn);
        if (cand.size() >= 8) break;
    }
    if (cand.empty()) cand.push_back((int)std::min<int64_t>(256, (M + 15) / 16 * 16));

    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    cudaEvent_t e0, e1;
    RTS_CUDA_TRY(ctx, cudaEventCreate(&e0));
    RTS_CUDA_TRY(ctx, cudaEventCreate(&e1));
    int best = 0;
    double best_t = 1e300;
    int n_tried = 0, rc = RTS_OK;
    for (int bn : cand) {
        rts_batch* b = nullptr;
        if ((rc = rts_batch_create(ctx, &b)) != RTS_OK) break;
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
        for (int w = 0; w < 2 && rc == RTS_OK; ++w) rc = rts_batch_step(b, 1);
        float ms = 0.0f;
        const int reps = 5;
        if (rc == RTS_OK) {
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps && rc == RTS_OK; ++r) rc = rts_batch_step(b, 1);
            cudaEventRecord(e1, st);
            if (rc == RTS_OK) rc = rts_batch_sync(b, 10000000);
            if (rc == RTS_OK) cudaEventElapsedTime(&ms, e0, e1);
        }
        rts_batch_destroy(b);
        if (rc != RTS_OK) break;
        const double t = ms / reps;
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
    rts_tune_entry* e = find_entry(ctx, M, precision, std::max(flush, 1));
    if (!e) {
        ctx->tune.push_back(rts_tune_entry());
        e = &ctx->tune.back();
    }
    *e = rts_tune_entry{M, precision, std::max(flush, 1), best, best_t};
    ctx->tuning_epoch++;
    return RTS_OK;
}

extern "C" int rts_autotune_save(rts_ctx* ctx, const char* path)
{
    if (!ctx || !path) return RTS_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "w");
    RTS_REQUIRE(ctx, f, RTS_ERR_INVALID_ARGUMENT, "cannot write %s", path);
    std::fprintf(f, "# rts tile-width table: M precision flush bn ms\n");
    for (const rts_tune_entry& e : ctx->tune)
        std::fprintf(f, "%lld %d %d %d %.6f\n", (long long)e.M, e.precision, e.flush, e.bn, e.ms);
    const bool ok = std::fclose(f) == 0;
    RTS_REQUIRE(ctx, ok, RTS_ERR_INVALID_ARGUMENT, "error writing %s", path);
    return RTS_OK;
}

extern "C" int rts_autotune_load(rts_ctx* ctx, const char* path)
{
    if (!ctx || !path) return RTS_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "r");
    RTS_REQUIRE(ctx, f, RTS_ERR_INVALID_ARGUMENT, "cannot read %s", path);
    char line[256];
    int n = 0, rc = RTS_OK;
    while (std::fgets(line, sizeof(line), f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        long long M = 0;
        int prec = 0, fl = 0, bn = 0;
        double ms = 0.0;
        if (std::sscanf(line, "%lld %d %d %d %lf", &M, &prec, &fl, &bn, &ms) != 5 || M < 1 ||
            (prec != RTS_PREC_FP16X3 && prec != RTS_PREC_BF16X3 && prec != RTS_PREC_TF32X3) || fl < 1 || fl > 2 ||
            bn < 16 || bn > 256 ||
            bn % 16 != 0) {
            rc = rts_fail(ctx, RTS_ERR_INVALID_ARGUMENT, "%s: malformed entry: %s", path, line);
            break;
        }
        rts_tune_entry* e = find_entry(ctx, M, prec, fl);
        if (!e) {
            ctx->tune.push_back(rts_tune_entry());
            e = &ctx->tune.back();
        }
        *e = rts_tune_entry{M, prec, fl, bn, ms};
        ++n;
    }
    std::fclose(f);
    if (rc == RTS_OK) ctx->tuning_epoch++;
    return rc;
}
