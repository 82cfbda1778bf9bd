// cuda_solve_compat.cpp -- the reference's GPU host interface
// (cuda/cuda_solve.h:5-37) implemented over the C ABI of librts_scatter.so.
//
// Drop-in use: compile this file into the reference's solver in place of
// cuda/cuda_solve.cu and cuda/cuda_struct.cu (with USE_CUDA defined, so that
// the reference's cuda/cuda_solve.h and solve_module/solve_global_struct.h
// provide grid_t, grid_directions_t and e_cuda_stream_id_t) and link
// librts_scatter.so.  The caller -- MPI_CalculateIllumAsync
// (solve_module/illum/Illum_async.cpp:616-1097), CalculateIllumParam (:1390),
// RunSolveModule (solve_module/solve_main.cpp:135-136,315) -- is unchanged.
//
// Behaviour kept from the reference: one process-wide device context created
// by SetDevice; InitDevice hands pinned host arrays to grid_t (Illum,
// scattering, and on the first rank the moment arrays); the Illum copies go on
// stream eCuda_scattering_1; every function returns 0 on success.
// Behaviour changed on purpose: errors are printed and reported with a return
// value of 1 (or, for void functions, remembered and printed) instead of
// exit(1) (cuda/cuda_def.cuh:14-20); the D2H of
// CalculateIntScatteringAsyncMPIStream lands at row `start` (start*N
// elements), where the reference offsets by `start` elements
// (cuda/cuda_solve.cu:107), which is the same for the start == 0 the solver
// uses; CalculateEnergy / CalculateStream / CalculateDivStream /
// CalculateDivImpuls compute their moments (their kernels are commented out
// in the reference, cuda/cuda_solve.cu:182,236,259).
//
// Precision: every call is FP64, bit-compatible with the reference, unless
// the RTS_SCATTER_PRECISION environment variable names a tensor-core
// precision (fp16x3, bf16x3 or tf32x3).  Then InitDevice sets that precision
// on the context (rts_set_precision) and every scattering call -- the
// asynchronous calls on the device-resident Illum that the source iteration
// makes (CalculateIntScatteringAsyncMPIStream, ...AsyncMPI, ...Async) and the
// synchronous CalculateIntScattering -- runs the split tcgen05 path, to
// <= 1e-6 relative for fp16x3 and tf32x3.  At a tensor precision the
// RTS_SCATTER_TUNE environment variable may name a schedule table file: when
// the file exists InitDevice loads it (rts_autotune_load); when it does not,
// InitDevice runs the schedule autotuner once for this rank's directions and
// cells (rts_autotune_schedule) and writes the table there, so later runs of
// the solver start from it.  The schedule changes the speed of the calls;
// within the accuracy above, not their results.
//
// Cell geometry: like the reference's InitDevice (cuda/cuda_struct.cu:134-176),
// the first rank reads normals.bin, squares.bin and volume.bin from the
// solver's base directory -- glb_files.base_adress when this file is built
// inside the reference (RTS_COMPAT_GLB_FILES defined, global_value.h
// included), otherwise the RTS_GEOMETRY_DIR environment variable (with a
// trailing separator, as base_adress has).  Missing files leave the
// divergence calls failing with a message, as in the reference.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "cuda_solve.h"
#include "rts_scatter.h"
#ifdef RTS_COMPAT_GLB_FILES
#include "global_value.h"
#endif

namespace {

rts_ctx* g_ctx = nullptr;
int g_device = 0;
bool g_owns_moments = false;

// RTS_SCATTER_PRECISION: fp64 (default), fp16x3, bf16x3 or tf32x3
int env_precision()
{
    const char* v = std::getenv("RTS_SCATTER_PRECISION");
    if (!v) return RTS_PREC_FP64;
    const std::string s(v);
    if (s == "fp16x3") return RTS_PREC_FP16X3;
    if (s == "bf16x3") return RTS_PREC_BF16X3;
    if (s == "tf32x3") return RTS_PREC_TF32X3;
    if (s != "fp64" && !s.empty())
        std::fprintf(stderr, "RTS_SCATTER_PRECISION=%s is not fp64, fp16x3, bf16x3 or tf32x3: using fp64\n", v);
    return RTS_PREC_FP64;
}

int report(int rc, const char* where)
{
    if (rc != RTS_OK)
        std::fprintf(stderr, "%s failed: status %d: %s\n", where, rc, g_ctx ? rts_last_error(g_ctx) : "");
    return rc == RTS_OK ? 0 : 1;
}

// RTS_SCATTER_TUNE: load the schedule table, or tune and write it
void tune_schedule(int precision, int M, int64_t cells)
{
    const char* path = std::getenv("RTS_SCATTER_TUNE");
    if (!path || !*path || precision == RTS_PREC_FP64) return;
    if (std::FILE* f = std::fopen(path, "r")) {
        std::fclose(f);
        report(rts_autotune_load(g_ctx, path), "InitDevice (schedule table)");
        return;
    }
    rts_tune_choice best;
    if (report(rts_autotune_schedule(g_ctx, M, precision, cells, &best, nullptr, 0, nullptr),
               "InitDevice (schedule autotuner)"))
        return;
    report(rts_autotune_save(g_ctx, path), "InitDevice (schedule table)");
}

rts_stream_id stream_of(e_cuda_stream_id_t s)
{
    switch (s) {
    case eCuda_scattering_1: return RTS_STREAM_SCATTERING_1;
    case eCuda_scattering_2: return RTS_STREAM_SCATTERING_2;
    default: return RTS_STREAM_PARAMS;
    }
}

std::string geometry_dir()
{
#ifdef RTS_COMPAT_GLB_FILES
    return glb_files.base_adress;
#else
    const char* d = std::getenv("RTS_GEOMETRY_DIR");
    return d ? std::string(d) : std::string();
#endif
}

// normals.bin: count-prefixed cells of four Vector3; squares.bin: 4 areas per
// cell; volume.bin: one volume per cell (file_module/reader_bin.cpp:49-69,
// reader_bin.h:13-30).
void load_geometry(int N)
{
    const std::string dir = geometry_dir();
    if (dir.empty()) return;
    std::vector<double> n((size_t)N * 12), s((size_t)N * 4), v((size_t)N);
    int64_t cn = 0, cs = 0, cv = 0;
    if (rts_read_simple_bin((dir + "normals.bin").c_str(), 96, N, n.data(), &cn) != RTS_OK ||
        rts_read_simple_bin((dir + "squares.bin").c_str(), 8, 4 * (int64_t)N, s.data(), &cs) != RTS_OK ||
        rts_read_simple_bin((dir + "volume.bin").c_str(), 8, N, v.data(), &cv) != RTS_OK || cn != N ||
        cs != 4 * (int64_t)N || cv != N) {
        std::fprintf(stderr, "InitDevice: cell geometry (normals.bin, squares.bin, volume.bin) not read from %s\n",
                     dir.c_str());
        return;
    }
    report(rts_set_geometry(g_ctx, n.data(), s.data(), v.data()), "InitDevice (geometry)");
}

int params(e_cuda_stream_id_t st, grid_t& grid, bool energy, bool stream, bool impuls, bool divstream,
           bool divimpuls, const char* where)
{
    return report(rts_illum_params(g_ctx, stream_of(st), energy ? grid.energy : nullptr,
                                   stream ? reinterpret_cast<double*>(grid.stream) : nullptr,
                                   impuls ? reinterpret_cast<double*>(grid.impuls) : nullptr,  // symmetric: either order
                                   divstream ? grid.divstream : nullptr,
                                   divimpuls ? reinterpret_cast<double*>(grid.divimpuls) : nullptr),
                  where);
}

}  // namespace

void SetDevice(const int num_dev)
{
    if (g_ctx) rts_ctx_destroy(g_ctx);
    g_ctx = nullptr;
    g_device = num_dev;
    report(rts_ctx_create(num_dev, &g_ctx), "SetDevice");
}

void InitDevice(const grid_directions_t& grid_dir_host, grid_t& grid_host, const int start, const int end)
{
    if (!g_ctx) SetDevice(g_device);
    if (!g_ctx) return;
    const int M = grid_dir_host.size;
    std::vector<double> xyz(3 * (size_t)M), area((size_t)M);
    for (int i = 0; i < M; ++i) {
        xyz[3 * i + 0] = grid_dir_host.directions[i].dir[0];
        xyz[3 * i + 1] = grid_dir_host.directions[i].dir[1];
        xyz[3 * i + 2] = grid_dir_host.directions[i].dir[2];
        area[i] = grid_dir_host.directions[i].area;
    }
    if (report(rts_init(g_ctx, xyz.data(), area.data(), M, grid_dir_host.full_area, grid_host.size, start, end),
               "InitDevice"))
        return;
    rts_host_illum(g_ctx, &grid_host.Illum);
    rts_host_scattering(g_ctx, &grid_host.scattering);
    const int precision = env_precision();
    if (report(rts_set_precision(g_ctx, precision), "InitDevice (precision)") == 0)
        tune_schedule(precision, M, grid_host.size);
    if (start == 0) {  // the first rank also receives the moments (cuda/cuda_struct.cu:158-175)
        grid_host.divstream = new Type[grid_host.size]();
        grid_host.divimpuls = new Vector3[grid_host.size]();
        grid_host.energy = new Type[grid_host.size]();
        grid_host.stream = new Vector3[grid_host.size]();
        grid_host.impuls = new Matrix3[grid_host.size]();
        g_owns_moments = true;
        load_geometry(grid_host.size);
    }
}

void ClearDevice()
{
    rts_ctx_destroy(g_ctx);  // frees the pinned Illum / scattering too
    g_ctx = nullptr;
}

void ClearHost(grid_t& grid_host)
{
    // Illum and scattering belong to the context (freed by ClearDevice)
    grid_host.Illum = nullptr;
    grid_host.scattering = nullptr;
    if (g_owns_moments) {
        delete[] grid_host.divstream;
        delete[] grid_host.divimpuls;
        delete[] grid_host.energy;
        delete[] grid_host.stream;
        delete[] grid_host.impuls;
        g_owns_moments = false;
    }
    grid_host.divstream = nullptr;
    grid_host.divimpuls = nullptr;
    grid_host.energy = nullptr;
    grid_host.stream = nullptr;
    grid_host.impuls = nullptr;
}

void CudaWait() { report(rts_wait(g_ctx, -1), "CudaWait"); }

void CudaSyncStream(const e_cuda_stream_id_t stream_id)
{
    report(rts_sync_stream(g_ctx, stream_of(stream_id), -1), "CudaSyncStream");
}

void CudaEventPrint()
{
    double ms = 0.0;
    int64_t n = 0;
    if (rts_kernel_timing(g_ctx, 0, &ms, &n) == RTS_OK && n > 0)
        std::printf("scattering kernels: %lld launches, %f ms total\n", (long long)n, ms);
    rts_kernel_timing(g_ctx, 1, nullptr, nullptr);
}

void CudaSendIllumAsync(const int size, const int shift, const Type* Illum_host)
{
    report(rts_send_illum_async(g_ctx, size, shift, shift, Illum_host), "CudaSendIllumAsync");
}

void CudaSendIllumAsync(const int size, const int shift_dev, const int shift_host, const Type* Illum_host)
{
    report(rts_send_illum_async(g_ctx, size, shift_dev, shift_host, Illum_host), "CudaSendIllumAsync");
}

void CopyIllumOnDevice(const int size, const Type* Illum_host)
{
    report(rts_copy_illum(g_ctx, size, Illum_host), "CopyIllumOnDevice");
}

int CalculateIntScatteringAsyncMPIStream(const grid_directions_t&, grid_t& grid, const int start, const int end,
                                         const e_cuda_stream_id_t stream)
{
    return report(rts_scattering_async(g_ctx, start, end, stream_of(stream), grid.scattering),
                  "CalculateIntScatteringAsyncMPIStream");
}

int CalculateIntScatteringAsyncMPI(const grid_directions_t&, grid_t& grid, int local_size)
{
    return report(rts_scattering_async(g_ctx, 0, local_size, RTS_STREAM_SCATTERING_1, grid.scattering),
                  "CalculateIntScatteringAsyncMPI");
}

int CalculateIntScatteringAsync(const grid_directions_t& grid_dir, grid_t& grid)
{
    return report(rts_scattering_async(g_ctx, 0, grid_dir.size, RTS_STREAM_SCATTERING_1, grid.scattering),
                  "CalculateIntScatteringAsync");
}

int CalculateIntScattering(const grid_directions_t&, grid_t& grid)
{
    return report(rts_scattering(g_ctx, grid.Illum, grid.scattering), "CalculateIntScattering");
}

int CalculateEnergy(const grid_directions_t&, grid_t& grid)
{
    return report(rts_moments(g_ctx, RTS_STREAM_PARAMS, grid.energy, nullptr), "CalculateEnergy");
}

int CalculateStream(const grid_directions_t&, grid_t& grid)
{
    return report(rts_moments(g_ctx, RTS_STREAM_PARAMS, nullptr, reinterpret_cast<double*>(grid.stream)),
                  "CalculateStream");
}

int CalculateImpuls(const grid_directions_t&, grid_t& grid)
{
    return params(eCuda_params, grid, false, false, true, false, false, "CalculateImpuls");
}

int CalculateDivImpuls(const grid_directions_t&, grid_t& grid)
{
    return params(eCuda_params, grid, false, false, grid.impuls != nullptr, false, true, "CalculateDivImpuls");
}

int CalculateDivStream(const grid_directions_t&, grid_t& grid)
{
    return params(eCuda_params, grid, false, grid.stream != nullptr, false, true, false, "CalculateDivStream");
}

int CalculateAllParam(const grid_directions_t& grid_dir, grid_t& grid)
{
    return CalculateAllParamStream(grid_dir, grid, eCuda_params);
}

int CalculateAllParamStream(const grid_directions_t&, grid_t& grid, e_cuda_stream_id_t st)
{
    // d_MakeIllumParam: the divergences (always), energy / flux / impulse when
    // the host arrays exist (CUDA_FULL_ARRAYS in the reference)
    return params(st, grid, grid.energy != nullptr, grid.stream != nullptr, grid.impuls != nullptr,
                  grid.divstream != nullptr, grid.divimpuls != nullptr, "CalculateAllParamStream");
}
