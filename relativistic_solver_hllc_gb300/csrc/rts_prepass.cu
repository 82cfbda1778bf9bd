// rts_prepass.cu -- operand preparation of the split-precision path.
//
// Every tensor-core contraction reads its operands as "interleaved split"
// rows: for FP16 / BF16, for each group of 32 in-directions 32 high parts
// followed by 32 low parts (16-bit, 128 bytes), x*scale = hi + lo; for TF32,
// for each group of 16 in-directions 16 high then 16 low parts (FP32 bit
// patterns, 128 bytes), no scale.  Sizes are in 16-bit units: a row holds
// 2*kpad of them (4*kpad for TF32).  The mode argument is 0 BF16, 1 FP16,
// 2 TF32.  These kernels build them:
//   * W^T rows (one per out-direction) from the FP64 direction-pair matrix,
//     with a power-of-two column scale in FP16 mode;
//   * Ibar rows (one per cell) from the reference's face-layout Illum
//     [M][N][4] FP64 (face mean in the reference's order, then split), or from
//     a direction-major FP32 Ibar [groups][M][N];
//   * per-row power-of-two scales (FP16 mode) putting max(|Ibar|, |B|) * 2
//     into [2^13, 2^14), so hi + lo keeps 22 bits with 4x headroom to 65504;
//   * the inverse (rows back to FP64 Ibar) for inspection.
// All are HBM-bound: the Illum prepass reads 32 B and writes 4 B per
// (cell, direction); its staged form reads the 32 B once, writes and reads
// back the 8 B FP64 face sum and writes the 4 B of rows.  Transposes go
// through shared memory so both the direction-major reads and the
// cell-major writes are coalesced.
#include <cstdint>

#include "rts_internal.h"
#include "rts_ptx.cuh"

using namespace rts_ptx;

namespace {

// 2^(13 - ilogb(m)), within FP32's normal range (rows or columns whose
// largest value is below 2^-113 or above 2^139 keep the nearest scale).
__device__ __forceinline__ float pow2_scale(double m)
{
    if (!(m > 0.0) || !isfinite(m)) return 1.0f;
    return ldexpf(1.0f, max(-126, min(127, 13 - ilogb(m))));
}

// Block sum of one double per thread (blockDim.x a multiple of 32); every
// thread receives the total.
__device__ double block_sum(double x, double* red)
{
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __syncthreads();  // red may still be read from a previous call
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    return t;
}

// Statistics of W [Min][ldw] FP64 (column k = out-direction, Mout == Min) for
// the conservation correction of relaxed steps, in v [kpad + 4] (FP32):
//   v[j] = sum_k W[j][k] (FP64 sums, k in order) for j < Min, 0 up to kpad;
//   v[kpad] the scale of the partial sums, 2^(7 - ceil(log2 sum_jk |W_jk|));
//   v[kpad+1] c, the FP32 value of the mean of the v_j; v[kpad+2] D, the sum
//   of d_j = v_j - c; v[kpad+3] 1 / c;
// and u [Min] FP64, u_i = sum_j W[i][j] d_j: the extra row of W^T whose
// output is sum_j d_j (W^T x)_j.  v64 [Min] FP64 scratch.  One block.
__global__ void __launch_bounds__(1024) w_stats_kernel(const double* __restrict__ W, int Min, int Mout, int ldw,
                                                       int kpad, float* __restrict__ v, double* __restrict__ v64,
                                                       double* __restrict__ u)
{
    __shared__ double red[32];
    double a = 0.0, sv = 0.0;
    for (int j = threadIdx.x; j < kpad; j += blockDim.x) {
        double s = 0.0;
        if (j < Min)
            for (int k = 0; k < Mout; ++k) {
                const double w = W[(int64_t)j * ldw + k];
                s += w;
                a += fabs(w);
            }
        v[j] = (float)s;
        if (j < Min) {
            v64[j] = s;
            sv += s;
        }
    }
    a = block_sum(a, red);
    sv = block_sum(sv, red);  // (its barriers also publish v64 to the block)
    const float c = Min > 0 ? (float)(sv / Min) : 0.0f;
    if (threadIdx.x == 0) {
        float q = 0.0f;
        if (a > 0.0 && isfinite(a)) {
            const int e = 7 - (int)ceil(log2(a));
            if (e > -126 && e < 127) q = ldexpf(1.0f, e);
        }
        v[kpad] = q;
        v[kpad + 1] = c;
        v[kpad + 3] = c != 0.0f ? 1.0f / c : 0.0f;
    }
    double ds = 0.0;
    for (int i = threadIdx.x; i < Min; i += blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < Mout; ++j) s += W[(int64_t)i * ldw + j] * (v64[j] - (double)c);
        u[i] = s;
        ds += v64[i] - (double)c;
    }
    ds = block_sum(ds, red);
    if (threadIdx.x == 0) v[kpad + 2] = (float)ds;
}

// W [Min][ldw] FP64 (column k = out-direction) -> Wc [mpad][2*kpad] split
// W^T rows; with `extra`, row Mout holds extra [Min] (the correction's row).
__global__ void split_w_kernel(const double* __restrict__ W, int Min, int Mout, int ldw, int kpad, int mpad,
                               int mode, uint16_t* __restrict__ Wc, float* __restrict__ cs,
                               const double* __restrict__ extra)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= mpad) return;
    const int units = (mode == 2 ? 4 : 2) * kpad;
    uint16_t* row = Wc + (int64_t)k * units;
    float* cs_inv = cs + mpad;
    // element j of this row: column k of W, or the extra row
    const bool ex = extra && k == Mout;
    const double* col = ex ? extra : W + k;
    const int64_t step = ex ? 1 : ldw;
    if (k >= Mout && !ex) {
        for (int j = 0; j < units; ++j) row[j] = 0;
        cs[k] = 1.0f;
        cs_inv[k] = 1.0f;
        return;
    }
    if (mode == 2) {
        float* rowf = reinterpret_cast<float*>(row);
        for (int j = 0; j < kpad; ++j) {
            float hi = 0.0f, lo = 0.0f;
            if (j < Min) split_tf32((float)col[j * step], hi, lo);
            rowf[ilv_hi_tf32(j)] = hi;
            rowf[ilv_hi_tf32(j) + 16] = lo;
        }
        cs[k] = 1.0f;
        cs_inv[k] = 1.0f;
        return;
    }
    const int fp16 = mode == 1;
    float s = 1.0f;
    if (fp16) {
        double m = 0.0;
        for (int j = 0; j < Min; ++j) m = fmax(m, fabs(col[j * step]));
        s = pow2_scale(m);
    }
    for (int j = 0; j < kpad; ++j) {
        uint16_t hi = 0, lo = 0;
        if (j < Min) split_any(fp16 != 0, (float)(col[j * step] * (double)s), hi, lo);
        row[ilv_hi(j)] = hi;
        row[ilv_hi(j) + 32] = lo;
    }
    cs[k] = s;
    cs_inv[k] = 1.0f / s;
}

__device__ __forceinline__ double face_mean(const double* __restrict__ illum, int64_t N, int j, int64_t c)
{
    const double2* p = reinterpret_cast<const double2*>(illum + ((int64_t)j * N + c) * 4);
    const double2 a = __ldg(p), b = __ldg(p + 1);
    double I = 0.0;  // faces 0..3 in order, then /4 (GET_FACE_TO_CELL)
    I += a.x;
    I += a.y;
    I += b.x;
    I += b.y;
    return I / 4;
}

// Row scales from the face layout: thread per cell.  The N cells are columns
// of an Illum whose rows hold `ld` cells (a cell range of a wider Illum).
__global__ void rowscale_faces_kernel(const double* __restrict__ illum, int64_t N, int64_t ld, int M,
                                      const double* __restrict__ B, float* __restrict__ rs, int64_t npad)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= npad) return;
    float s = 1.0f;
    if (c < N) {
        double m = B ? fabs(B[c]) : 0.0;
        for (int j = 0; j < M; ++j) m = fmax(m, fabs(face_mean(illum, ld, j, c)));
        s = pow2_scale(2.0 * m);
    }
    rs[c] = s;
    rs[npad + c] = 1.0f / s;
}

// x * 2^k rounded to the nearest FP32 (ties to even), from the bit pattern
// on the integer pipe: GB300's FP64 pipe issues about two instructions per SM
// per cycle against 128 for FP32 / integer, and would bound a pass that
// scaled and converted every value there.  Where x * 2^k is in FP32's normal
// range the 52-bit mantissa keeps its top 23 bits, rounded on the 29 below
// (a carry into the exponent is the correctly rounded result, up to
// infinity); zeros, FP64 subnormals, FP32 subnormal or overflowing results
// and NaN take ldexp and the hardware conversion.  Either way one rounding
// of the exact product.
__device__ __forceinline__ float pow2_scaled_to_f32(double x, int k)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((u >> 52) & 0x7FF);
    const int ef = e + k - 1023 + 127;  // biased FP32 exponent of x * 2^k
    if (e == 0 || e == 0x7FF || ef < 1 || ef > 254) return __double2float_rn(ldexp(x, k));
    const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
    unsigned int f = ((unsigned int)ef << 23) | (unsigned int)(m >> 29);
    const unsigned int rem = (unsigned int)m & 0x1FFFFFFFu;
    if (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ++f;
    return __uint_as_float(f | ((unsigned int)(u >> 32) & 0x80000000u));
}

// Face sums of the face layout (FP64, the reference's order) into a
// direction-major staging [M][N], and with cmax non-null the per-cell max
// over the directions of |face sum| (FP64 bits: non-negative doubles order
// like unsigned integers, so the max runs on the integer pipe and merges with
// atomicMax; NaN is skipped, as fmax does in the row-scale pass above).  The
// FP64 work is the 3 adds of the sum.  Thread per (cell, 32 directions): a
// warp reads 1 KB and writes 256 B contiguous per direction, no transpose.
__global__ void __launch_bounds__(256) face_sums_kernel(const double* __restrict__ illum, int64_t N, int64_t ld,
                                                        int jb, int je, double* __restrict__ sums,
                                                        unsigned long long* __restrict__ cmax)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int j0 = jb + blockIdx.y * 32;  // directions [jb, je) of the launch, 32 per block row
    const int j1 = min(je, j0 + 32);
    unsigned long long mx = 0;
#pragma unroll 8
    for (int j = j0; j < j1; ++j) {
        const double2* p = reinterpret_cast<const double2*>(illum + ((int64_t)j * ld + c) * 4);
        const double2 a = __ldg(p), b = __ldg(p + 1);
        double I = a.x;  // faces 0..3 in order (GET_FACE_TO_CELL), as face_mean
        I += a.y;
        I += b.x;
        I += b.y;
        sums[(int64_t)j * N + c] = I;
        const unsigned long long ub = (unsigned long long)__double_as_longlong(I) & 0x7FFFFFFFFFFFFFFFull;
        if (ub <= 0x7FF0000000000000ull && ub > mx) mx = ub;
    }
    if (cmax) atomicMax(cmax + c, mx);
}

// Row scales from the per-cell maxima of face_sums_kernel: the scale of
// rowscale_faces_kernel (max_j |sum / 4| = max_j |sum| / 4 exactly; max is
// order-free).
__global__ void rowscale_from_max_kernel(const unsigned long long* __restrict__ cmax, int64_t N,
                                         const double* __restrict__ B, float* __restrict__ rs, int64_t npad)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= npad) return;
    float s = 1.0f;
    if (c < N) {
        const double m = B ? fabs(B[c]) : 0.0;
        s = pow2_scale(2.0 * fmax(m, __longlong_as_double((long long)cmax[c]) / 4));
    }
    rs[c] = s;
    rs[npad + c] = 1.0f / s;
}

// Row scales from direction-major FP32 Ibar [groups][M][N]: thread per row.
__global__ void rowscale_f32_kernel(const float* __restrict__ ibar, int64_t N, int M, int64_t rows,
                                    const float* __restrict__ B, float* __restrict__ rs, int64_t rows_pad)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows_pad) return;
    float s = 1.0f;
    if (r < rows) {
        const int64_t g = r / N, c = r - g * N;
        const float* base = ibar + g * (int64_t)M * N + c;
        double m = B ? fabs((double)B[r]) : 0.0;
        for (int j = 0; j < M; ++j) m = fmax(m, fabs((double)base[(int64_t)j * N]));
        s = pow2_scale(2.0 * m);
    }
    rs[r] = s;
    rs[rows_pad + r] = 1.0f / s;
}

// x * s rounded once to FP32 (s a power of two): an FP64 source multiplies
// in FP64, an FP32 one in FP32 -- the same exact product, one rounding, and
// no FP64 instruction for the FP32 sources.
__device__ __forceinline__ float scaled_f32(double x, float s) { return (float)(x * (double)s); }
__device__ __forceinline__ float scaled_f32(float x, float s) { return x * s; }
// A staged face sum: its mean x / 4 times s, by the exponent arithmetic above
// (s a normal power of two).
struct FaceSum {
    double x;
};
__device__ __forceinline__ float scaled_f32(FaceSum v, float s)
{
    return pow2_scaled_to_f32(v.x, (int)((__float_as_uint(s) >> 23) & 0xFF) - 127 - 2);
}

// Transpose-and-split through shared memory.  Tile: 32 in-directions x 64
// rows, 256 threads.  `Src` supplies the value of (direction j, row r).
template <class Src>
__device__ __forceinline__ void split_tile(const Src& src, int64_t rows, int M, int kpad, const float* __restrict__ rs,
                                           int mode, uint16_t* __restrict__ A)
{
    __shared__ float tile[64][33];
    const int j0 = blockIdx.y * 32;
    const int64_t r0 = (int64_t)blockIdx.x * 64;
    const int t = threadIdx.x;
    {
        const int rr = t & 63;
        const int64_t r = r0 + rr;
        const float s = (r < rows && rs) ? rs[r] : 1.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int jj = (t >> 6) + 4 * q;
            const int j = j0 + jj;
            tile[rr][jj] = (r < rows && j < M) ? scaled_f32(src(j, r), s) : 0.0f;
        }
    }
    __syncthreads();
    const int rr = t >> 2;
    const int part = t & 3;  // 0,1: hi of j 0-15 / 16-31; 2,3: lo of j 0-15 / 16-31
    const int64_t r = r0 + rr;
    if (r >= rows) return;
    const int jbase = (part & 1) * 16;
    if (mode == 2) {
        // TF32: the 32 in-directions are two 16-wide groups; part 0/1 the
        // high parts of group 0/1, part 2/3 their low parts (64 B each)
        float out[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            float hi, lo;
            split_tf32(tile[rr][jbase + i], hi, lo);
            out[i] = (part < 2) ? hi : lo;
        }
        float* dst = reinterpret_cast<float*>(A + r * 4 * (int64_t)kpad) + (int64_t)((j0 >> 4) + (part & 1)) * 32 +
                     (part >= 2 ? 16 : 0);
        float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
        for (int i = 0; i < 4; ++i) d4[i] = make_float4(out[4 * i], out[4 * i + 1], out[4 * i + 2], out[4 * i + 3]);
        return;
    }
    const int fp16 = mode == 1;
    uint16_t out[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        uint16_t hi, lo;
        split_any(fp16 != 0, tile[rr][jbase + i], hi, lo);
        out[i] = (part < 2) ? hi : lo;
    }
    uint16_t* dst = A + r * 2 * (int64_t)kpad + (int64_t)(j0 >> 5) * 64 + (part >= 2 ? 32 : 0) + jbase;
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    d4[0] = make_uint4(pack2(out[0], out[1]), pack2(out[2], out[3]), pack2(out[4], out[5]), pack2(out[6], out[7]));
    d4[1] = make_uint4(pack2(out[8], out[9]), pack2(out[10], out[11]), pack2(out[12], out[13]),
                       pack2(out[14], out[15]));
}

struct FacesSrc {
    const double* illum;
    int64_t N;
    __device__ double operator()(int j, int64_t c) const { return face_mean(illum, N, j, c); }
};

struct F32Src {
    const float* ibar;
    int64_t N;
    int M;
    __device__ float operator()(int j, int64_t r) const
    {
        const int64_t g = r / N, c = r - g * N;
        return __ldg(ibar + (g * M + j) * N + c);
    }
};

// The direction-major FP64 face sums of face_sums_kernel.
struct SumSrc {
    const double* sums;
    int64_t N;
    __device__ FaceSum operator()(int j, int64_t c) const { return FaceSum{__ldg(sums + (int64_t)j * N + c)}; }
};

__global__ void __launch_bounds__(256) split_sums_kernel(const double* __restrict__ sums, int64_t N, int M, int kpad,
                                                         const float* __restrict__ rs, int mode,
                                                         uint16_t* __restrict__ A)
{
    split_tile(SumSrc{sums, N}, N, M, kpad, rs, mode, A);
}

__global__ void __launch_bounds__(256) split_faces_kernel(const double* __restrict__ illum, int64_t N, int64_t ld,
                                                          int M, int kpad, const float* __restrict__ rs, int mode,
                                                          uint16_t* __restrict__ A)
{
    split_tile(FacesSrc{illum, ld}, N, M, kpad, rs, mode, A);
}

__global__ void __launch_bounds__(256) split_f32_kernel(const float* __restrict__ ibar, int64_t N, int M,
                                                        int64_t rows, int kpad, const float* __restrict__ rs,
                                                        int mode, uint16_t* __restrict__ A)
{
    split_tile(F32Src{ibar, N, M}, rows, M, kpad, rs, mode, A);
}

// Rows back to direction-major FP64 Ibar [groups][M][N].
__global__ void join_rows_kernel(const uint16_t* __restrict__ A, int64_t N, int M, int64_t rows, int kpad,
                                 const float* __restrict__ rs_inv, int mode, double* __restrict__ out)
{
    const int64_t total = (int64_t)M * rows;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        // i enumerates [g][j][c]
        const int64_t g = i / ((int64_t)M * N);
        const int64_t rem = i - g * (int64_t)M * N;
        const int64_t j = rem / N, c = rem - j * N;
        const int64_t r = g * N + c;
        float x;
        if (mode == 2) {
            const float* rowf = reinterpret_cast<const float*>(A + r * 4 * (int64_t)kpad);
            x = rowf[ilv_hi_tf32(j)] + rowf[ilv_hi_tf32(j) + 16];
        } else {
            const uint16_t* row = A + r * 2 * (int64_t)kpad;
            x = join_any(mode == 1, row[ilv_hi(j)], row[ilv_hi(j) + 32]);
        }
        out[i] = (double)x * (double)(rs_inv ? rs_inv[r] : 1.0f);
    }
}

__global__ void f32_to_f64_kernel(const float* __restrict__ s, double* __restrict__ d, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (double)s[i];
}

__global__ void f64_to_f32_kernel(const double* __restrict__ s, float* __restrict__ d, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (float)s[i];
}

int blocks_for(rts_ctx* ctx, int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)ctx->num_sms * 16;
    return (int)(b > cap ? cap : (b < 1 ? 1 : b));
}

}  // namespace

int rts_pp_w_stats(rts_ctx* ctx, const double* W, int Min, int Mout, int ldw, int kpad, float* v, double* v64,
                   double* u, cudaStream_t st)
{
    w_stats_kernel<<<1, 1024, 0, st>>>(W, Min, Mout, ldw, kpad, v, v64, u);
    RTS_CHECK_LAUNCH(ctx, "w_stats_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_pp_split_w(rts_ctx* ctx, const double* W, int Min, int Mout, int ldw, int kpad, int mpad, int mode,
                   uint16_t* Wc, float* cs, cudaStream_t st, const double* extra)
{
    split_w_kernel<<<(mpad + 127) / 128, 128, 0, st>>>(W, Min, Mout, ldw, kpad, mpad, mode, Wc, cs, extra);
    RTS_CHECK_LAUNCH(ctx, "split_w_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_pp_rows_from_faces(rts_ctx* ctx, const double* illum, int64_t N, int64_t ld, int M, int kpad, const double* B,
                           int mode, float* rs, int64_t npad, uint16_t* A, cudaStream_t st, bool bound)
{
    const bool fp16 = mode == 1;
    if (fp16 || bound) {  // the scales; the unscaled formats keep them only as a bound of the rows
        rowscale_faces_kernel<<<(unsigned)((npad + 127) / 128), 128, 0, st>>>(illum, N, ld, M, B, rs, npad);
        RTS_CHECK_LAUNCH(ctx, "rowscale_faces_kernel");
        ctx->launches++;
    }
    dim3 grid((unsigned)((N + 63) / 64), (unsigned)(kpad / 32));
    split_faces_kernel<<<grid, 256, 0, st>>>(illum, N, ld, M, kpad, fp16 ? rs : nullptr, mode, A);
    RTS_CHECK_LAUNCH(ctx, "split_faces_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_pp_face_sums(rts_ctx* ctx, const double* illum, int64_t N, int64_t ld, int j0, int j1, double* sums,
                     unsigned long long* cmax, cudaStream_t st)
{
    if (j1 <= j0) return RTS_OK;
    face_sums_kernel<<<dim3((unsigned)((N + 255) / 256), (unsigned)((j1 - j0 + 31) / 32)), 256, 0, st>>>(
        illum, N, ld, j0, j1, sums, cmax);
    RTS_CHECK_LAUNCH(ctx, "face_sums_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_pp_rows_from_faces_staged(rts_ctx* ctx, const double* illum, int64_t N, int64_t ld, int M, int kpad,
                                  const double* B, int mode, float* rs, int64_t npad, uint16_t* A, double* sums,
                                  unsigned long long* cmax, cudaStream_t st, bool bound)
{
    const bool scaled = mode == 1 || bound;
    if (scaled) RTS_CUDA_TRY(ctx, cudaMemsetAsync(cmax, 0, (size_t)N * sizeof(unsigned long long), st));
    int rc = rts_pp_face_sums(ctx, illum, N, ld, 0, M, sums, scaled ? cmax : nullptr, st);
    if (rc != RTS_OK) return rc;
    return rts_pp_rows_from_sums(ctx, N, M, kpad, B, mode, rs, npad, A, sums, cmax, st, bound);
}

int rts_pp_rows_from_sums(rts_ctx* ctx, int64_t N, int M, int kpad, const double* B, int mode, float* rs, int64_t npad,
                          uint16_t* A, const double* sums, const unsigned long long* cmax, cudaStream_t st, bool bound)
{
    const bool fp16 = mode == 1;
    const bool scaled = fp16 || bound;
    if (scaled) {
        rowscale_from_max_kernel<<<(unsigned)((npad + 127) / 128), 128, 0, st>>>(cmax, N, B, rs, npad);
        RTS_CHECK_LAUNCH(ctx, "rowscale_from_max_kernel");
        ctx->launches++;
    }
    dim3 grid((unsigned)((N + 63) / 64), (unsigned)(kpad / 32));
    split_sums_kernel<<<grid, 256, 0, st>>>(sums, N, M, kpad, fp16 ? rs : nullptr, mode, A);
    RTS_CHECK_LAUNCH(ctx, "split_sums_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_pp_rows_from_f32(rts_ctx* ctx, const float* ibar, int64_t N, int M, int64_t rows, int kpad, const float* B,
                         int mode, float* rs, int64_t rows_pad, uint16_t* A, cudaStream_t st, bool bound)
{
    const bool fp16 = mode == 1;
    if (fp16 || bound) {
        rowscale_f32_kernel<<<(unsigned)((rows_pad + 127) / 128), 128, 0, st>>>(ibar, N, M, rows, B, rs, rows_pad);
        RTS_CHECK_LAUNCH(ctx, "rowscale_f32_kernel");
        ctx->launches++;
    }
    dim3 grid((unsigned)((rows + 63) / 64), (unsigned)(kpad / 32));
    split_f32_kernel<<<grid, 256, 0, st>>>(ibar, N, M, rows, kpad, fp16 ? rs : nullptr, mode, A);
    RTS_CHECK_LAUNCH(ctx, "split_f32_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_pp_join_rows(rts_ctx* ctx, const uint16_t* A, int64_t N, int M, int64_t rows, int kpad, const float* rs_inv,
                     int mode, double* out, cudaStream_t st)
{
    join_rows_kernel<<<blocks_for(ctx, (int64_t)M * rows, 256), 256, 0, st>>>(A, N, M, rows, kpad, rs_inv, mode, out);
    RTS_CHECK_LAUNCH(ctx, "join_rows_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_pp_f32_to_f64(rts_ctx* ctx, const float* s, double* d, int64_t n, cudaStream_t st)
{
    f32_to_f64_kernel<<<blocks_for(ctx, n, 256), 256, 0, st>>>(s, d, n);
    RTS_CHECK_LAUNCH(ctx, "f32_to_f64_kernel");
    ctx->launches++;
    return RTS_OK;
}

int rts_pp_f64_to_f32(rts_ctx* ctx, const double* s, float* d, int64_t n, cudaStream_t st)
{
    f64_to_f32_kernel<<<blocks_for(ctx, n, 256), 256, 0, st>>>(s, d, n);
    RTS_CHECK_LAUNCH(ctx, "f64_to_f32_kernel");
    ctx->launches++;
    return RTS_OK;
}
