// rts_solution.cpp -- the radiation part of the reference's solution dump
// (WriteFileSolution, file_module/writer_bin.cpp:15-44, CUDA build) from the
// device-resident state: Illum.bin (the face mean of direction 0 per cell,
// GetDirectionIllumFromFace, solve_module/illum/illum_utils.cpp:11-28),
// energy.bin, stream.bin, impuls.bin, and with the cell geometry divstream.bin
// and divimpuls.bin.  Every file is an int32 count followed by the raw
// elements (WRITE_FILE, global_def.h:212-220): N doubles, N x 3 doubles for
// the vectors, N x 9 for the (symmetric) impulse tensor.
#include <climits>
#include <cstdio>
#include <string>
#include <vector>

#include "rts_internal.h"

namespace {

std::string join(const char* dir, const char* name)
{
    std::string d(dir);
    if (!d.empty() && d.back() != '/') d += '/';
    return d + name;
}

int write_counted(rts_ctx* ctx, const std::string& path, int n, const double* data, int per_cell)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    RTS_REQUIRE(ctx, f, RTS_ERR_INVALID_ARGUMENT, "cannot write %s", path.c_str());
    bool ok = std::fwrite(&n, sizeof(int), 1, f) == 1;
    ok = ok && std::fwrite(data, sizeof(double) * (size_t)per_cell, (size_t)n, f) == (size_t)n;
    ok = (std::fclose(f) == 0) && ok;
    RTS_REQUIRE(ctx, ok, RTS_ERR_INVALID_ARGUMENT, "error writing %s", path.c_str());
    return RTS_OK;
}

}  // namespace

extern "C" int rts_write_solution(rts_ctx* ctx, const char* dir)
{
    if (!ctx || !dir) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_write_solution before rts_init");
    const int64_t N = ctx->N;
    RTS_REQUIRE(ctx, N <= INT_MAX, RTS_ERR_UNSUPPORTED, "%lld cells do not fit the files' int32 count",
                (long long)N);
    const bool div = ctx->d_geo != nullptr;
    std::vector<double> energy((size_t)N), flux((size_t)N * 3), impuls((size_t)N * 9);
    std::vector<double> divstream(div ? (size_t)N : 0), divimpuls(div ? (size_t)N * 3 : 0);
    int rc = rts_illum_params(ctx, RTS_STREAM_PARAMS, energy.data(), flux.data(), impuls.data(),
                              div ? divstream.data() : nullptr, div ? divimpuls.data() : nullptr);
    if (rc != RTS_OK) return rc;
    // direction 0 of the face layout, averaged over the four faces in order
    std::vector<double> faces((size_t)N * 4), illum((size_t)N);
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(faces.data(), ctx->d_illum, rts_bytes<double>(N * 4), cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    for (int64_t c = 0; c < N; ++c) {
        double I = 0.0;
        for (int f = 0; f < 4; ++f) I += faces[(size_t)(c * 4 + f)];
        illum[(size_t)c] = I / 4;
    }
    const int n = (int)N;
    if ((rc = write_counted(ctx, join(dir, "Illum.bin"), n, illum.data(), 1)) != RTS_OK) return rc;
    if ((rc = write_counted(ctx, join(dir, "energy.bin"), n, energy.data(), 1)) != RTS_OK) return rc;
    if ((rc = write_counted(ctx, join(dir, "stream.bin"), n, flux.data(), 3)) != RTS_OK) return rc;
    if ((rc = write_counted(ctx, join(dir, "impuls.bin"), n, impuls.data(), 9)) != RTS_OK) return rc;
    if (div) {
        if ((rc = write_counted(ctx, join(dir, "divstream.bin"), n, divstream.data(), 1)) != RTS_OK) return rc;
        if ((rc = write_counted(ctx, join(dir, "divimpuls.bin"), n, divimpuls.data(), 3)) != RTS_OK) return rc;
    }
    return RTS_OK;
}
