// rts_flush.cpp -- the automatic drain period of the tensor-core path.
//
// tcgen05.mma rounds each FP32 accumulate toward zero.  Within a drain
// period (a chunk of `flush` K-slices, two hi*hi MMAs of 16 in-directions
// per slice) every MMA that follows the one carrying most of an output's
// value truncates about one to two ulps of that value again; the drain into
// round-to-nearest FP32 registers ends the chain.  With two K-slices per
// drain an output dominated by one 16-direction block can lose up to three
// such truncations more than with one, ~5e-7 of itself in FP16x3 -- too much
// of a 1e-6 budget.  So two slices per drain are used only when no
// 16-direction block of any out-direction's column of W carries more than
// 1/8 of the column (then the extra loss stays below ~7e-8): smooth kernels
// (Thomson, Henyey-Greenstein with small g) on enough directions.  Peaked
// kernels, small direction sets and caller-supplied W drain every slice.
//
// TF32x3 slices hold 16 in-directions (kind::tf32 multiplies 8 per MMA), so
// its drain count per in-direction is twice FP16's at the same period, and
// the round-to-nearest FP32 additions of the drains -- a random walk of
// about sqrt(drains)/6 ulps of the sum -- dominate its error instead; it
// drains every two slices (32 in-directions, the FP16x3 setting for peaked
// kernels), measured within 1e-6 on peaked and smooth kernels alike where
// one slice per drain reached 1.1e-6 at M = 1202.
#include <cmath>
#include <cstdint>
#include <vector>

#include "rts_internal.h"

int rts_auto_flush(const double* xyz, const double* area, int64_t M, double full_area, int64_t k0, int64_t k1,
                   int phase, double g, int precision)
{
    if (precision == RTS_PREC_TF32X3) return 2;
    if (phase != RTS_PHASE_THOMSON && phase != RTS_PHASE_HG) return 1;
    if (!xyz || !area || M <= 0 || k1 <= k0) return 1;
    const double pi = 3.14159265358979323846264338327950288;
    constexpr int SAMPLES = 16;
    std::vector<double> w((size_t)M);
    double worst = 0.0;
    for (int s = 0; s < SAMPLES; ++s) {
        const int64_t k = k0 + (k1 - k0 - 1) * s / (SAMPLES - 1);
        const double bx = xyz[3 * k], by = xyz[3 * k + 1], bz = xyz[3 * k + 2];
        double col = 0.0;
        for (int64_t j = 0; j < M; ++j) {
            const double mu = xyz[3 * j] * bx + xyz[3 * j + 1] * by + xyz[3 * j + 2] * bz;
            double v;
            if (phase == RTS_PHASE_THOMSON) {
                v = 0.75 * (1.0 + mu * mu) * area[j] / full_area;
            } else {
                const double den = 1.0 + g * g - 2.0 * g * mu;
                v = area[j] * (1.0 - g * g) / (4.0 * pi * den * std::sqrt(den));
            }
            w[(size_t)j] = std::fabs(v);
            col += w[(size_t)j];
        }
        if (!(col > 0.0)) return 1;
        for (int64_t j0 = 0; j0 < M; j0 += 16) {
            double b = 0.0;
            for (int64_t j = j0; j < j0 + 16 && j < M; ++j) b += w[(size_t)j];
            if (b / col > worst) worst = b / col;
        }
    }
    return worst <= 0.125 ? 2 : 1;
}
