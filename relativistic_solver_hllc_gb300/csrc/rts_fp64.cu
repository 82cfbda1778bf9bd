// rts_fp64.cu -- FP64 CUDA-core kernels of the scattering path:
//   * the plain FP64 scattering integral (replaces d_GetS / d_GetS_MPI /
//     d_GetS_MPI_Stream, cuda/cuda_kernel.cu:23-111), with the source update
//     and the FP64 residual fused into its epilogue;
//   * the direction-pair weights W (Gamma of cuda/cuda_utils.cu:7-16 times
//     area_j / full_area, or renormalised Henyey-Greenstein);
//   * FP64 energy and flux moments (cuda/cuda_utils.cu:18-67,
//     cuda/cuda_kernel.cu:113-134) in one pass over Illum;
//   * standalone source update / residual and the FP64 relaxation step;
//   * the synthetic lognormal Illum generator.
//
// The reference kernel gives each thread one (cell, out-direction) pair and
// loops over all in-directions, re-reading the 4 faces and recomputing Gamma
// for every pair and accumulating straight into global memory.  Here a CTA
// owns a 128-cell x 64-out-direction tile (the out-directions left over
// past a multiple of 64 take one narrower tile): the face mean is taken once per
// (in-direction, cell) while the tile of Ibar is staged in shared memory, W
// (FP64, precomputed once) is staged beside it, and each thread keeps an
// 8-cell x 4-direction block of accumulators in registers.  GB300 FP64 runs
// at a small fraction of its FP32 rate, so this kernel is FP64-pipe bound by
// design; memory traffic is ~40 B per cell-direction pair over M in-directions.
#include <cstdint>
#include <mutex>

#include "rts_internal.h"

namespace {

constexpr int F64_TC = 128;  // cells per CTA
constexpr int F64_TK = 64;   // out-directions per CTA
constexpr int F64_KC = 16;   // in-directions per shared-memory chunk
constexpr int F64_THREADS = 256;

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Residual bits: non-negative doubles order the same as their bit patterns.
__device__ __forceinline__ void residual_max(unsigned long long* dst, double v)
{
    v = warp_max(v);
    if ((threadIdx.x & 31) == 0 && v > 0.0)
        atomicMax(dst, (unsigned long long)__double_as_longlong(v));
}

// One tile of 128 cells x 16*NB out-directions [k0, k0 + 16*NB): each
// thread keeps 8 cells x NB directions of accumulators.  Every output is the
// same FMA chain over the in-directions in order whatever NB, so a tile's
// width changes no result.  GB300's FP64 pipe retires about two FMAs per SM
// per cycle, far below the shared-memory loads that feed them, so a narrow
// tile costs about NB/4 of a full one.
template <bool kUpdate, bool kResidual, int NB>
__device__ __forceinline__ void scatter_tile(double (*sI)[F64_TC], double (*sW)[F64_TK],
                                             const double* __restrict__ illum, const double* __restrict__ W,
                                             int64_t N, int M, int ldw, int k0, int k_end, double* __restrict__ S,
                                             const double* __restrict__ B, double lambda,
                                             unsigned long long* __restrict__ resid)
{
    constexpr int TK = 16 * NB;
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t c0 = (int64_t)blockIdx.x * F64_TC;

    double acc[NB][8];
#pragma unroll
    for (int m = 0; m < NB; ++m)
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[m][i] = 0.0;

    for (int j0 = 0; j0 < M; j0 += F64_KC) {
        // Ibar chunk: F64_KC x 128 (in-direction, cell) pairs, 8 per thread;
        // consecutive threads read consecutive cells' 32-byte face groups.
#pragma unroll
        for (int q = 0; q < (F64_KC * F64_TC) / F64_THREADS; ++q) {
            const int p = tid + F64_THREADS * q;
            const int jj = p / F64_TC, cc = p % F64_TC;
            const int j = j0 + jj;
            const int64_t c = c0 + cc;
            double v = 0.0;
            if (j < M && c < N) {
                const double2* src = reinterpret_cast<const double2*>(illum + ((int64_t)j * N + c) * 4);
                const double2 a = __ldg(src), b = __ldg(src + 1);
                double I = 0.0;  // faces 0..3 in order, then /4 (GET_FACE_TO_CELL)
                I += a.x;
                I += a.y;
                I += b.x;
                I += b.y;
                v = I / 4;
            }
            sI[jj][cc] = v;
        }
        // W chunk: F64_KC x TK, NB per thread
#pragma unroll
        for (int q = 0; q < (F64_KC * TK) / F64_THREADS; ++q) {
            const int p = tid + F64_THREADS * q;
            const int jj = p / TK, kk = p % TK;
            const int j = j0 + jj, k = k0 + kk;
            sW[jj][kk] = (j < M && k < k_end) ? __ldg(W + (int64_t)j * ldw + k) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < F64_KC; ++jj) {
            double iv[8], wv[NB];
#pragma unroll
            for (int i = 0; i < 8; ++i) iv[i] = sI[jj][tx + 16 * i];
#pragma unroll
            for (int m = 0; m < NB; ++m) wv[m] = sW[jj][ty + 16 * m];
#pragma unroll
            for (int m = 0; m < NB; ++m)
#pragma unroll
                for (int i = 0; i < 8; ++i) acc[m][i] = fma(wv[m], iv[i], acc[m][i]);
        }
        __syncthreads();
    }

    double rmax = 0.0;
#pragma unroll
    for (int m = 0; m < NB; ++m) {
        const int k = k0 + ty + 16 * m;
        if (k >= k_end) continue;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t c = c0 + tx + 16 * i;
            if (c >= N) continue;
            double v = acc[m][i];
            if (kUpdate) v = (1.0 - lambda) * B[c] + lambda * v;
            double* dst = S + (int64_t)k * N + c;
            if (kResidual) rmax = fmax(rmax, fabs(v - *dst));
            *dst = v;
        }
    }
    if (kResidual) residual_max(resid, rmax);
}

// Grid: x over 128-cell tiles; y over the out-directions [k_begin, k_end),
// n_full tiles of 64 and then, when the range is not a multiple of 64, one
// tile of 16*nb_last (nb_last 1..4) for the rest.  The narrow tiles are last
// in launch order, so they fill the final wave.
template <bool kUpdate, bool kResidual>
__global__ void __launch_bounds__(F64_THREADS)
scatter_fp64_kernel(const double* __restrict__ illum, const double* __restrict__ W, int64_t N,
                    int M, int ldw, int k_begin, int k_end, int n_full, int nb_last, double* __restrict__ S,
                    const double* __restrict__ B, double lambda,
                    unsigned long long* __restrict__ resid)
{
    __shared__ double sI[F64_KC][F64_TC];
    __shared__ double sW[F64_KC][F64_TK];
    const int k0 = k_begin + (int)blockIdx.y * F64_TK;
    const int nb = (int)blockIdx.y < n_full ? 4 : nb_last;
    switch (nb) {
    case 1:
        scatter_tile<kUpdate, kResidual, 1>(sI, sW, illum, W, N, M, ldw, k0, k_end, S, B, lambda, resid);
        break;
    case 2:
        scatter_tile<kUpdate, kResidual, 2>(sI, sW, illum, W, N, M, ldw, k0, k_end, S, B, lambda, resid);
        break;
    case 3:
        scatter_tile<kUpdate, kResidual, 3>(sI, sW, illum, W, N, M, ldw, k0, k_end, S, B, lambda, resid);
        break;
    default:
        scatter_tile<kUpdate, kResidual, 4>(sI, sW, illum, W, N, M, ldw, k0, k_end, S, B, lambda, resid);
        break;
    }
}

// The y extent of scatter_fp64_kernel's grid over `width` out-directions.
struct DirTiles {
    int n_full, nb_last, gy;
};
inline DirTiles dir_tiles(int64_t width)
{
    DirTiles t;
    t.n_full = (int)(width / F64_TK);
    const int rem = (int)(width % F64_TK);
    t.nb_last = rem ? (rem + 15) / 16 : 4;
    t.gy = t.n_full + (rem ? 1 : 0);
    return t;
}

__device__ __forceinline__ double gamma_thomson(double ax, double ay, double az, double bx,
                                                double by, double bz)
{
    double dot = 0.0;  // x, y, z order as cuda/cuda_utils.cu:7-16
    dot += ax * bx;
    dot += ay * by;
    dot += az * bz;
    return (3. * (1 + dot * dot)) / 4;
}

// One thread per local out-direction column of W [M][loc].
__global__ void weights_kernel(const double* __restrict__ xyz, const double* __restrict__ area,
                               int M, int k_off, int loc, double full_area, int phase, double g,
                               double* __restrict__ W)
{
    const int kl = blockIdx.x * blockDim.x + threadIdx.x;
    if (kl >= loc) return;
    const int k = k_off + kl;
    const double bx = xyz[3 * k], by = xyz[3 * k + 1], bz = xyz[3 * k + 2];
    if (phase == RTS_PHASE_THOMSON) {
        for (int j = 0; j < M; ++j)
            W[(int64_t)j * loc + kl] =
                gamma_thomson(xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], bx, by, bz) * area[j] /
                full_area;
        return;
    }
    const double pi = 3.14159265358979323846264338327950288;
    double colsum = 0.0;
    for (int j = 0; j < M; ++j) {
        const double mu = xyz[3 * j] * bx + xyz[3 * j + 1] * by + xyz[3 * j + 2] * bz;
        const double den = 1.0 + g * g - 2.0 * g * mu;
        const double kv = (1.0 - g * g) / (4.0 * pi * den * sqrt(den));
        const double w = area[j] * kv;
        W[(int64_t)j * loc + kl] = w;
        colsum += w;
    }
    for (int j = 0; j < M; ++j) W[(int64_t)j * loc + kl] /= colsum;
}

constexpr int MOM_THREADS = 128;
constexpr int MOM_DCHUNK = 256;

// Energy and flux of every cell in one pass over Illum (FP64).  Per
// direction the shared table holds area_j / 4 and w_j area_j / 4, so a
// (cell, direction) costs the face sum (3 adds) and four FMAs -- the
// reference's sum_j (sum_f I_f / 4) area_j w_j regrouped, the FP64 pipe
// being the bound.
__global__ void __launch_bounds__(MOM_THREADS)
moments_kernel(const double* __restrict__ illum, const double* __restrict__ xyz,
               const double* __restrict__ area, int64_t N, int M, double full_area,
               double* __restrict__ energy, double* __restrict__ flux)
{
    __shared__ double sd[MOM_DCHUNK][4];
    const int64_t c = (int64_t)blockIdx.x * MOM_THREADS + threadIdx.x;
    double e = 0.0, fx = 0.0, fy = 0.0, fz = 0.0;
    for (int j0 = 0; j0 < M; j0 += MOM_DCHUNK) {
        const int nj = min(MOM_DCHUNK, M - j0);
        for (int t = threadIdx.x; t < nj; t += MOM_THREADS) {
            const double a4 = area[j0 + t] * 0.25;  // exact
            sd[t][0] = a4;
            sd[t][1] = xyz[3 * (j0 + t)] * a4;
            sd[t][2] = xyz[3 * (j0 + t) + 1] * a4;
            sd[t][3] = xyz[3 * (j0 + t) + 2] * a4;
        }
        __syncthreads();
        if (c < N) {
            for (int jj = 0; jj < nj; ++jj) {
                const double2* src =
                    reinterpret_cast<const double2*>(illum + ((int64_t)(j0 + jj) * N + c) * 4);
                const double2 a = __ldg(src), b = __ldg(src + 1);
                const double sum = ((a.x + a.y) + b.x) + b.y;
                e = fma(sum, sd[jj][0], e);
                fx = fma(sum, sd[jj][1], fx);
                fy = fma(sum, sd[jj][2], fy);
                fz = fma(sum, sd[jj][3], fz);
            }
        }
        __syncthreads();
    }
    if (c < N) {
        energy[c] = e / full_area;
        flux[3 * c] = fx / full_area;
        flux[3 * c + 1] = fy / full_area;
        flux[3 * c + 2] = fz / full_area;
    }
}

// Energy, flux, impulse tensor and the divergences of flux and impulse of
// every cell in one pass over Illum (FP64).  The reference computes them in
// d_MakeIllumParam (cuda/cuda_kernel.cu:218-223: d_MakeEnergy :113-121,
// d_MakeDivStream :149-175, d_MakeDivImpuls :177-216) with per-face sums
// (cuda/cuda_utils.cu:86-167).  Here the per-face sums are never formed: with
// ia_f = I[j][c][f] * area_j and the face vectors nS_f = n_f * S_f,
//   flux      = sum_j w_j * (sum_f ia_f) / (4 full_area)
//   impuls    = sum_j w_j w_j^T * (sum_f ia_f) / (4 full_area)
//   divstream = sum_j (w_j . u_j) / (full_area V),   u_j = sum_f ia_f nS_f
//   divimpuls = sum_j w_j (w_j . u_j) / (full_area V)
// which are the reference's sums regrouped (the same terms, other order).
// The direction's area rides in the shared table (area_j, area_j w_j and
// area_j w_j w_j^T), so the face intensities are summed once and scaled by
// no per-cell multiply: 32 FP64 operations per (cell, direction) instead of
// the reference's 80.
constexpr int PAR_THREADS = 128;
constexpr int PAR_DCHUNK = 128;

__global__ void __launch_bounds__(PAR_THREADS)
illum_params_kernel(const double* __restrict__ illum, const double* __restrict__ xyz,
                    const double* __restrict__ area, int64_t N, int M, double full_area,
                    const double* __restrict__ normals, const double* __restrict__ face_areas,
                    const double* __restrict__ volume, double* __restrict__ out)
{
    // per direction: area, area w (3), area w w^T (xx, xy, xz, yy, yz, zz), w (3)
    __shared__ double sd[PAR_DCHUNK][13];
    const int64_t c = (int64_t)blockIdx.x * PAR_THREADS + threadIdx.x;
    const bool geo = normals != nullptr;
    double nS[4][3];
#pragma unroll
    for (int f = 0; f < 4; ++f)
#pragma unroll
        for (int d = 0; d < 3; ++d)
            nS[f][d] = (geo && c < N) ? normals[c * 12 + 3 * f + d] * face_areas[c * 4 + f] : 0.0;
    double e = 0.0, fl[3] = {0.0, 0.0, 0.0}, im[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    double ds = 0.0, di[3] = {0.0, 0.0, 0.0};
    for (int j0 = 0; j0 < M; j0 += PAR_DCHUNK) {
        const int nj = min(PAR_DCHUNK, M - j0);
        for (int t = threadIdx.x; t < nj; t += PAR_THREADS) {
            const double x = xyz[3 * (j0 + t)], y = xyz[3 * (j0 + t) + 1], z = xyz[3 * (j0 + t) + 2];
            const double a = area[j0 + t];
            sd[t][0] = a;
            sd[t][1] = a * x, sd[t][2] = a * y, sd[t][3] = a * z;
            sd[t][4] = a * (x * x), sd[t][5] = a * (x * y), sd[t][6] = a * (x * z);
            sd[t][7] = a * (y * y), sd[t][8] = a * (y * z), sd[t][9] = a * (z * z);
            sd[t][10] = x, sd[t][11] = y, sd[t][12] = z;
        }
        __syncthreads();
        if (c < N) {
            for (int jj = 0; jj < nj; ++jj) {
                const double2* src =
                    reinterpret_cast<const double2*>(illum + ((int64_t)(j0 + jj) * N + c) * 4);
                const double2 p = __ldg(src), q = __ldg(src + 1);
                const double sum = ((p.x + p.y) + q.x) + q.y;
                e = fma(sd[jj][0], sum, e);
#pragma unroll
                for (int d = 0; d < 3; ++d) fl[d] = fma(sd[jj][1 + d], sum, fl[d]);
#pragma unroll
                for (int d = 0; d < 6; ++d) im[d] = fma(sd[jj][4 + d], sum, im[d]);
                if (geo) {
                    // u = sum_f I_f nS_f; area_j w_j . u, and w_j times it
                    double u[3];
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        u[d] = fma(q.y, nS[3][d], fma(q.x, nS[2][d], fma(p.y, nS[1][d], p.x * nS[0][d])));
                    const double s = fma(sd[jj][3], u[2], fma(sd[jj][2], u[1], sd[jj][1] * u[0]));
                    ds += s;
#pragma unroll
                    for (int d = 0; d < 3; ++d) di[d] = fma(sd[jj][10 + d], s, di[d]);
                }
            }
        }
        __syncthreads();
    }
    if (c >= N) return;
    const double q4 = 1.0 / (4.0 * full_area);
    double* o = out;  // [energy N][flux 3N][impuls 9N][divstream N][divimpuls 3N]
    o[c] = e * q4;
    o += N;
#pragma unroll
    for (int d = 0; d < 3; ++d) o[3 * c + d] = fl[d] * q4;
    o += 3 * N;
    const double t[9] = {im[0], im[1], im[2], im[1], im[3], im[4], im[2], im[4], im[5]};
#pragma unroll
    for (int d = 0; d < 9; ++d) o[9 * c + d] = t[d] * q4;
    o += 9 * N;
    if (geo) {
        const double qv = 1.0 / (full_area * volume[c]);
        o[c] = ds * qv;
        o += N;
#pragma unroll
        for (int d = 0; d < 3; ++d) o[3 * c + d] = di[d] * qv;
    }
}

template <bool kResidual>
__global__ void update_kernel(double* __restrict__ S, const double* __restrict__ B, int64_t N,
                              int64_t rows, double lambda, unsigned long long* __restrict__ resid)
{
    double rmax = 0.0;
    const int64_t total = rows * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double old = S[i];
        const double v = (1.0 - lambda) * B[i % N] + lambda * old;
        if (kResidual) rmax = fmax(rmax, fabs(v - old));
        S[i] = v;
    }
    if (kResidual) residual_max(resid, rmax);
}

// Illum[j][c][f] <- 0.5 Illum[j][c][f] + 0.5 S[j][c]
__global__ void relax_fp64_kernel(double* __restrict__ illum, const double* __restrict__ S,
                                  int64_t total_pairs)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total_pairs;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double s = S[i];
        double2* p = reinterpret_cast<double2*>(illum + i * 4);
        double2 a = p[0], b = p[1];
        a.x = 0.5 * a.x + 0.5 * s;
        a.y = 0.5 * a.y + 0.5 * s;
        b.x = 0.5 * b.x + 0.5 * s;
        b.y = 0.5 * b.y + 0.5 * s;
        p[0] = a;
        p[1] = b;
    }
}

// Counter hash shared with the CPU generator (splitmix64 finaliser).
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double uniform01(uint64_t key, uint64_t idx)
{
    const uint64_t r = mix64(key ^ mix64(idx));
    return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

__global__ void synth_illum_kernel(double* __restrict__ illum, int64_t pairs, uint64_t key,
                                   double mu, double sigma, int independent_faces)
{
    const double two_pi = 6.283185307179586476925286766559;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < pairs;
         i += (int64_t)gridDim.x * blockDim.x) {
        double v[4];
        if (independent_faces) {
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                const uint64_t idx = (uint64_t)i * 4 + f;
                const double u1 = uniform01(key, 2 * idx), u2 = uniform01(key, 2 * idx + 1);
                v[f] = exp(mu + sigma * (sqrt(-2.0 * log(u1)) * cos(two_pi * u2)));
            }
        } else {
            const uint64_t idx = (uint64_t)i;
            const double u1 = uniform01(key, 2 * idx), u2 = uniform01(key, 2 * idx + 1);
            v[0] = v[1] = v[2] = v[3] = exp(mu + sigma * (sqrt(-2.0 * log(u1)) * cos(two_pi * u2)));
        }
        double2* p = reinterpret_cast<double2*>(illum + i * 4);
        p[0] = make_double2(v[0], v[1]);
        p[1] = make_double2(v[2], v[3]);
    }
}

uint64_t host_mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int grid_stride_blocks(rts_ctx* ctx, int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)ctx->num_sms * 16;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

int rts_launch_scatter_fp64(rts_ctx* ctx, int64_t k_begin, int64_t k_end, cudaStream_t st,
                            const double* B, double lambda, bool update, bool residual)
{
    if (k_end <= k_begin) return RTS_OK;
    const int64_t gx = (ctx->N + F64_TC - 1) / F64_TC;
    const DirTiles dt = dir_tiles(k_end - k_begin);
    RTS_REQUIRE(ctx, gx < (1ll << 31) && dt.gy < 65536, RTS_ERR_UNSUPPORTED, "FP64 grid too large");
    dim3 grid((unsigned)gx, (unsigned)dt.gy);
    const int ldw = (int)ctx->local();
    rts_timing_begin(ctx, st);
    if (update && residual)
        scatter_fp64_kernel<true, true><<<grid, F64_THREADS, 0, st>>>(
            ctx->d_illum, ctx->d_W, ctx->N, (int)ctx->M, ldw, (int)k_begin, (int)k_end, dt.n_full, dt.nb_last,
            ctx->d_S, B, lambda, ctx->resid_target);
    else if (update)
        scatter_fp64_kernel<true, false><<<grid, F64_THREADS, 0, st>>>(
            ctx->d_illum, ctx->d_W, ctx->N, (int)ctx->M, ldw, (int)k_begin, (int)k_end, dt.n_full, dt.nb_last,
            ctx->d_S, B, lambda, ctx->resid_target);
    else
        scatter_fp64_kernel<false, false><<<grid, F64_THREADS, 0, st>>>(
            ctx->d_illum, ctx->d_W, ctx->N, (int)ctx->M, ldw, (int)k_begin, (int)k_end, dt.n_full, dt.nb_last,
            ctx->d_S, nullptr, 0.0, ctx->resid_target);
    rts_timing_end(ctx, st);
    RTS_CHECK_LAUNCH(ctx, "scatter_fp64_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_launch_weights(rts_ctx* ctx)
{
    const int loc = (int)ctx->local();
    weights_kernel<<<(loc + 127) / 128, 128, 0, ctx->streams[RTS_STREAM_SCATTERING_1]>>>(
        ctx->d_xyz, ctx->d_area, (int)ctx->M, (int)ctx->out_start, loc, ctx->full_area, ctx->phase,
        ctx->phase_g, ctx->d_W);
    RTS_CHECK_LAUNCH(ctx, "weights_kernel");
    ctx->launches++;
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->streams[RTS_STREAM_SCATTERING_1]));
    return RTS_OK;
}

int rts_launch_moments(rts_ctx* ctx, cudaStream_t st)
{
    const int64_t blocks = (ctx->N + MOM_THREADS - 1) / MOM_THREADS;
    rts_timing_begin(ctx, st);
    moments_kernel<<<(unsigned)blocks, MOM_THREADS, 0, st>>>(ctx->d_illum, ctx->d_xyz, ctx->d_area,
                                                             ctx->N, (int)ctx->M, ctx->full_area,
                                                             ctx->d_energy, ctx->d_flux);
    rts_timing_end(ctx, st);
    RTS_CHECK_LAUNCH(ctx, "moments_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_launch_illum_params(rts_ctx* ctx, cudaStream_t st)
{
    const int64_t blocks = (ctx->N + PAR_THREADS - 1) / PAR_THREADS;
    const double* geo = ctx->d_geo;
    const int64_t N = ctx->N;
    rts_timing_begin(ctx, st);
    illum_params_kernel<<<(unsigned)blocks, PAR_THREADS, 0, st>>>(
        ctx->d_illum, ctx->d_xyz, ctx->d_area, N, (int)ctx->M, ctx->full_area, geo, geo ? geo + 12 * N : nullptr,
        geo ? geo + 16 * N : nullptr, ctx->d_params);
    rts_timing_end(ctx, st);
    RTS_CHECK_LAUNCH(ctx, "illum_params_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_launch_update(rts_ctx* ctx, int64_t k_begin, int64_t k_end, cudaStream_t st,
                      const double* B, double lambda, bool residual)
{
    const int64_t rows = k_end - k_begin;
    if (rows <= 0) return RTS_OK;
    const int blocks = grid_stride_blocks(ctx, rows * ctx->N, 256);
    double* S = ctx->d_S + k_begin * ctx->N;
    if (residual)
        update_kernel<true><<<blocks, 256, 0, st>>>(S, B, ctx->N, rows, lambda, ctx->resid_target);
    else
        update_kernel<false><<<blocks, 256, 0, st>>>(S, B, ctx->N, rows, lambda, ctx->resid_target);
    RTS_CHECK_LAUNCH(ctx, "update_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_launch_relax_fp64(rts_ctx* ctx, cudaStream_t st)
{
    const int64_t pairs = ctx->M * ctx->N;
    relax_fp64_kernel<<<grid_stride_blocks(ctx, pairs, 256), 256, 0, st>>>(ctx->d_illum, ctx->d_S,
                                                                           pairs);
    RTS_CHECK_LAUNCH(ctx, "relax_fp64_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_launch_synth(rts_ctx* ctx, uint64_t seed, double mu, double sigma, int independent_faces)
{
    const int64_t pairs = ctx->M * ctx->N;
    const uint64_t key = host_mix64(seed * 0x632BE59BD9B4E019ull + 1);
    synth_illum_kernel<<<grid_stride_blocks(ctx, pairs, 256), 256, 0,
                         ctx->streams[RTS_STREAM_SCATTERING_1]>>>(ctx->d_illum, pairs, key, mu, sigma,
                                                                  independent_faces);
    RTS_CHECK_LAUNCH(ctx, "synth_illum_kernel");
    ctx->launches++;
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->streams[RTS_STREAM_SCATTERING_1]));
    return RTS_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free FP64 scattering integral.
//
// For callers that cannot allocate device memory themselves or through us:
// code running under a caller-owned memory pool or arena that forbids
// allocations outside it, and hosts that account every device byte up
// front.  The caller passes device inputs and outputs; the only scratch --
// the M x M FP64 direction-pair matrix W -- lives in the file-scope array
// below, which every GPU that loads this library holds until the process
// exits.
// ---------------------------------------------------------------------------
namespace {

static __device__ __align__(256) double g_noalloc_w[RTS_NOALLOC_MAX_DIRS * RTS_NOALLOC_MAX_DIRS];

constexpr int NOALLOC_MAX_DEVICES = 64;
double* g_noalloc_w_addr[NOALLOC_MAX_DEVICES] = {};
std::mutex g_noalloc_mutex;

// Device address of the scratch array for `device` (current).  Host code
// cannot use the symbol itself as a pointer, so the address is looked up with
// cudaGetSymbolAddress.  Outside a stream capture it is looked up on every
// call, so a module reloaded after a device reset is seen at its new address;
// the last address found is kept for calls made while `st` is being captured,
// which must therefore follow an uncaptured call on the same device.
double* noalloc_scratch(int device, cudaStream_t st)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return nullptr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (cap != cudaStreamCaptureStatusNone) return g_noalloc_w_addr[device];
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_w) != cudaSuccess) {
        cudaGetLastError();  // our own lookup's error; none was pending on entry
        return nullptr;
    }
    g_noalloc_w_addr[device] = static_cast<double*>(p);
    return g_noalloc_w_addr[device];
}

bool aligned(const void* p, uintptr_t bytes) { return (reinterpret_cast<uintptr_t>(p) & (bytes - 1)) == 0; }

}  // namespace

extern "C" int rts_scattering_noalloc(const double* d_illum, const double* d_xyz, const double* d_area,
                                      int64_t N, int64_t M, double full_area, double* d_scattering,
                                      void* stream)
{
    if (!d_illum || !d_xyz || !d_area || !d_scattering) return RTS_ERR_INVALID_ARGUMENT;
    if (N <= 0 || M <= 0 || !(full_area > 0.0)) return RTS_ERR_INVALID_ARGUMENT;
    if (M > RTS_NOALLOC_MAX_DIRS) return RTS_ERR_INVALID_ARGUMENT;  // the scratch holds M <= 512
    // Illum is read as pairs of doubles (16-byte loads); the rest as doubles
    if (!aligned(d_illum, 16) || !aligned(d_xyz, 8) || !aligned(d_area, 8) || !aligned(d_scattering, 8))
        return RTS_ERR_INVALID_ARGUMENT;
    const int64_t gx = (N + F64_TC - 1) / F64_TC;
    if (gx >= (1ll << 31)) return RTS_ERR_INVALID_ARGUMENT;
    // An error left pending by the caller's own earlier work is theirs: report
    // it without launching and without clearing it.
    if (cudaPeekAtLastError() != cudaSuccess) return RTS_ERR_CUDA;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return RTS_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double* W = noalloc_scratch(device, st);
    if (!W) return RTS_ERR_CUDA;
    // W is rewritten in full (all M x M entries) by every call: nothing in the
    // scratch has to start at zero, and calls that overlap on the GPU race.
    weights_kernel<<<(unsigned)((M + 127) / 128), 128, 0, st>>>(d_xyz, d_area, (int)M, 0, (int)M, full_area,
                                                                RTS_PHASE_THOMSON, 0.0, W);
    if (cudaGetLastError() != cudaSuccess) return RTS_ERR_CUDA;  // nothing was pending: this launch's error
    const DirTiles dt = dir_tiles(M);
    dim3 grid((unsigned)gx, (unsigned)dt.gy);
    scatter_fp64_kernel<false, false><<<grid, F64_THREADS, 0, st>>>(d_illum, W, N, (int)M, (int)M, 0, (int)M,
                                                                     dt.n_full, dt.nb_last, d_scattering, nullptr,
                                                                     0.0, nullptr);
    if (cudaGetLastError() != cudaSuccess) return RTS_ERR_CUDA;
    return RTS_OK;
}

// W [M][loc] of an arbitrary direction set on `st` (used by the batched path).
int rts_launch_weights_raw(rts_ctx* ctx, const double* d_xyz, const double* d_area, int M, int k_off, int loc,
                           double full_area, int phase, double g, double* W, cudaStream_t st)
{
    weights_kernel<<<(loc + 127) / 128, 128, 0, st>>>(d_xyz, d_area, M, k_off, loc, full_area, phase, g, W);
    RTS_CHECK_LAUNCH(ctx, "weights_kernel");
    ctx->launches++;
    return RTS_OK;
}
