// rts_io.cpp -- host-side formats and bookkeeping of the scattering path:
//   * the direction-set text file (ReadSphereDirectionDecartToSpherical,
//     file_module/reader_txt.cpp:25-47): M, then M lines "area x y z", then
//     full_area;
//   * count-prefixed binary arrays (ReadSimpleFileBin / WriteSimpleFileBin,
//     file_module/reader_bin.h:13-30, file_module/writer_bin.h:9-26): an int32
//     element count followed by the raw elements -- the layout of Illum.bin,
//     energy.bin, ... written by WriteFileSolution (file_module/writer_bin.cpp:15-44);
//   * the out-direction partition over ranks (GetSend / GetDisp,
//     solve_module/solve_utils.cpp:177-202).
// None of these touch the GPU.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "rts_scatter.h"

extern "C" {

int rts_read_direction_file(const char* path, int64_t capacity, int64_t* M, double* xyz, double* area,
                            double* full_area)
{
    if (!path || !M) return RTS_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "r");
    if (!f) return RTS_ERR_INVALID_ARGUMENT;
    long long n = 0;
    if (fscanf(f, "%lld", &n) != 1 || n <= 0 || n > (1ll << 24)) {
        fclose(f);
        return RTS_ERR_INVALID_ARGUMENT;
    }
    *M = n;
    if (!xyz || !area || capacity < n) {  // size query
        fclose(f);
        return RTS_OK;
    }
    for (long long i = 0; i < n; ++i) {
        if (fscanf(f, "%lf %lf %lf %lf", &area[i], &xyz[3 * i], &xyz[3 * i + 1], &xyz[3 * i + 2]) != 4) {
            fclose(f);
            return RTS_ERR_INVALID_ARGUMENT;
        }
    }
    double fa = 0.0;
    const int got = fscanf(f, "%lf", &fa);
    fclose(f);
    if (got != 1) return RTS_ERR_INVALID_ARGUMENT;
    if (full_area) *full_area = fa;
    return RTS_OK;
}

int rts_write_direction_file(const char* path, int64_t M, const double* xyz, const double* area,
                             double full_area)
{
    if (!path || M <= 0 || !xyz || !area) return RTS_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "w");
    if (!f) return RTS_ERR_INVALID_ARGUMENT;
    fprintf(f, "%lld\n", (long long)M);
    for (int64_t i = 0; i < M; ++i)
        fprintf(f, "%.17g %.17g %.17g %.17g\n", area[i], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    fprintf(f, "%.17g\n", full_area);
    const int bad = ferror(f);
    fclose(f);
    return bad ? RTS_ERR_INVALID_ARGUMENT : RTS_OK;
}

int rts_read_simple_bin(const char* path, int64_t elem_size, int64_t capacity, void* data, int64_t* count)
{
    if (!path || !count || elem_size <= 0) return RTS_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "rb");
    if (!f) return RTS_ERR_INVALID_ARGUMENT;
    int32_t n = 0;
    if (fread(&n, sizeof(n), 1, f) != 1 || n < 0) {
        fclose(f);
        return RTS_ERR_INVALID_ARGUMENT;
    }
    *count = n;
    if (!data || capacity < n) {  // size query
        fclose(f);
        return RTS_OK;
    }
    const size_t got = fread(data, (size_t)elem_size, (size_t)n, f);
    fclose(f);
    return got == (size_t)n ? RTS_OK : RTS_ERR_INVALID_ARGUMENT;
}

int rts_write_simple_bin(const char* path, int64_t elem_size, int64_t count, const void* data)
{
    if (!path || elem_size <= 0 || count < 0 || count > INT32_MAX || (count > 0 && !data))
        return RTS_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "wb");
    if (!f) return RTS_ERR_INVALID_ARGUMENT;
    const int32_t n = (int32_t)count;
    size_t ok = fwrite(&n, sizeof(n), 1, f);
    if (count > 0) ok += fwrite(data, (size_t)elem_size, (size_t)count, f) == (size_t)count ? 1 : 0;
    fclose(f);
    return ok == (count > 0 ? 2u : 1u) ? RTS_OK : RTS_ERR_INVALID_ARGUMENT;
}

int rts_partition(int np, int64_t n, int64_t* send, int64_t* disp)
{
    if (np <= 0 || n < 0 || !send || !disp) return RTS_ERR_INVALID_ARGUMENT;
    // counts: n / np each, the first n % np ranks one more
    for (int i = 0; i < np; ++i) send[i] = n / np + (i < n % np ? 1 : 0);
    // displacements: prefix sums of the counts (GetDisp computes the same
    // offsets by a closed form)
    disp[0] = 0;
    for (int i = 1; i < np; ++i) disp[i] = disp[i - 1] + send[i - 1];
    return RTS_OK;
}

}  // extern "C"
