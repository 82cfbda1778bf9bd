// rts_synth.cpp -- host-side synthetic-workload helpers of the C ABI:
// spherical Fibonacci direction sets (the direction-file layout of
// file_module/reader_txt.cpp:25-47: area, x, y, z per direction, then
// full_area) and counter-hash uniform values.  Benchmark inputs only; the
// device generator of lognormal intensities lives in rts_fp64.cu.
#include <cmath>
#include <cstdint>

#include "rts_scatter.h"

namespace {
uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
}  // namespace

extern "C" {

int rts_synth_directions(int64_t M, double* xyz, double* area, double* full_area)
{
    if (M <= 0 || !xyz || !area || !full_area) return RTS_ERR_INVALID_ARGUMENT;
    const double pi = 3.14159265358979323846264338327950288;
    const double golden = pi * (3.0 - std::sqrt(5.0));
    for (int64_t i = 0; i < M; ++i) {
        const double z = 1.0 - (2.0 * (double)i + 1.0) / (double)M;
        const double r = std::sqrt(std::fmax(0.0, 1.0 - z * z));
        const double phi = golden * (double)i;
        xyz[3 * i + 0] = r * std::cos(phi);
        xyz[3 * i + 1] = r * std::sin(phi);
        xyz[3 * i + 2] = z;
        area[i] = 4.0 * pi / (double)M;
    }
    *full_area = 4.0 * pi;
    return RTS_OK;
}

int rts_synth_uniform(uint64_t seed, uint64_t stream, double lo, double hi, int64_t i0, int64_t n,
                      double* out)
{
    if (n < 0 || (n > 0 && !out)) return RTS_ERR_INVALID_ARGUMENT;
    const uint64_t key = mix64(seed * 0x632BE59BD9B4E019ull + stream);
    for (int64_t i = 0; i < n; ++i) {
        const uint64_t r = mix64(key ^ mix64((uint64_t)(i0 + i)));
        const double u = ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        out[i] = lo + (hi - lo) * u;
    }
    return RTS_OK;
}

}  // extern "C"
