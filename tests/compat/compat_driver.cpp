// compat_driver.cpp -- calls the reference-named GPU interface
// (cuda_solve_compat.cpp) in the order of the reference's source iteration
// (solve_module/illum/Illum_async.cpp): SetDevice + InitDevice, per-direction
// CudaSendIllumAsync, the two CalculateIntScatteringAsyncMPIStream launches
// of :1019-1020 on streams 1 and 2, CudaSyncStream, CalculateAllParamStream,
// then the synchronous CalculateIntScattering, ClearDevice and ClearHost.
// Inputs/outputs are files (direction text file, count-prefixed binaries) so
// a test can compare them with the oracle.
//   compat_driver <dirs.txt> <Illum.bin> <N> <outdir>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cuda_solve.h"
#include "rts_scatter.h"

static int fail(const char* m)
{
    std::fprintf(stderr, "compat_driver: %s\n", m);
    return 1;
}

int main(int argc, char** argv)
{
    if (argc != 5) return fail("usage: compat_driver dirs.txt Illum.bin N outdir");
    const std::string out = argv[4];
    const int N = std::atoi(argv[3]);
    int64_t M = 0;
    if (rts_read_direction_file(argv[1], 0, &M, nullptr, nullptr, nullptr) != RTS_OK) return fail("dirs");
    std::vector<double> xyz(3 * M), area(M);
    double fa = 0;
    if (rts_read_direction_file(argv[1], M, &M, xyz.data(), area.data(), &fa) != RTS_OK) return fail("dirs");
    grid_directions_t dirs;
    dirs.size = (int)M;
    dirs.directions.resize(M);
    for (int i = 0; i < M; ++i) {
        for (int d = 0; d < 3; ++d) dirs.directions[i].dir[d] = xyz[3 * i + d];
        dirs.directions[i].area = area[i];
    }
    dirs.full_area = fa;

    grid_t grid;
    grid.size = N;
    SetDevice(0);
    InitDevice(dirs, grid, 0, (int)M);
    if (!grid.Illum || !grid.scattering) return fail("InitDevice gave no host arrays");
    int64_t cnt = 0;
    if (rts_read_simple_bin(argv[2], 8, M * N * 4, grid.Illum, &cnt) != RTS_OK || cnt != M * N * 4)
        return fail("Illum.bin");

    const int size_1 = (int)M / 3;
    for (int j = 0; j < M; ++j) CudaSendIllumAsync(4 * N, 4 * N * j, grid.Illum);
    if (CalculateIntScatteringAsyncMPIStream(dirs, grid, 0, size_1, eCuda_scattering_1)) return fail("stream 1");
    if (CalculateIntScatteringAsyncMPIStream(dirs, grid, 0, (int)M, eCuda_scattering_2)) return fail("stream 2");
    CudaSyncStream(eCuda_scattering_1);
    CudaSyncStream(eCuda_scattering_2);
    rts_write_simple_bin((out + "/scattering.bin").c_str(), 8, M * N, grid.scattering);

    if (CalculateAllParamStream(dirs, grid, eCuda_params)) return fail("CalculateAllParamStream");
    CudaSyncStream(eCuda_params);
    rts_write_simple_bin((out + "/energy.bin").c_str(), 8, N, grid.energy);
    rts_write_simple_bin((out + "/stream.bin").c_str(), 24, N, grid.stream);
    rts_write_simple_bin((out + "/impuls.bin").c_str(), 72, N, grid.impuls);
    rts_write_simple_bin((out + "/divstream.bin").c_str(), 8, N, grid.divstream);
    rts_write_simple_bin((out + "/divimpuls.bin").c_str(), 24, N, grid.divimpuls);
    // the single-moment calls write the same arrays
    std::memset(grid.divstream, 0, sizeof(double) * N);
    if (CalculateDivStream(dirs, grid)) return fail("CalculateDivStream");
    if (CalculateDivImpuls(dirs, grid)) return fail("CalculateDivImpuls");
    if (CalculateImpuls(dirs, grid)) return fail("CalculateImpuls");
    rts_write_simple_bin((out + "/divstream2.bin").c_str(), 8, N, grid.divstream);

    std::memset(grid.scattering, 0, sizeof(double) * M * N);
    if (CalculateIntScattering(dirs, grid)) return fail("CalculateIntScattering");
    rts_write_simple_bin((out + "/scattering_sync.bin").c_str(), 8, M * N, grid.scattering);
    CudaWait();
    ClearDevice();
    ClearHost(grid);
    std::printf("compat_driver ok\n");
    return 0;
}
