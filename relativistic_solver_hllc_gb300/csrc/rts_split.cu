// rts_split.cu -- split-precision tensor-core path of the scattering integral
// (tcgen05 / TMEM / TMA, sm_103a).
//
// The integral S[k][c] = sum_j W[j][k] Ibar[j][c] is a dense contraction
// D = A B^T with A = Ibar^T (cells x in-directions) and B = W^T
// (out-directions x in-directions), both K-major.  Each operand is split into
// a 16-bit high part and a 16-bit low part (x = hi + lo + O(2^-22 x) for FP16
// with power-of-two row / column scaling, O(2^-17 x) for BF16) and the
// contraction runs the three products hi*hi + hi*lo + lo*hi on the tensor
// cores with FP32 accumulation in tensor memory.
//
// Operand layout in HBM ("interleaved split"): a row holds, for every group of
// 32 in-directions, 32 high halves followed by 32 low halves (128 bytes), so
// one 64-element TMA box with 128-byte swizzle brings both parts of a K-slice
// into shared memory and the three products address them at byte offsets 0 /
// 64 inside the same swizzle atom.
//
// Kernel (rts_split_gemm.cuh): one CTA per 128-cell x BN-out-direction tile
// (BN <= 256), 320 threads: warp 0 issues TMA loads into a 4-stage ring,
// warp 1 owns TMEM (hi*hi and cross-term accumulators) and issues tcgen05.mma
// from one thread, warps 2-9 drain TMEM (tcgen05.ld 32x32b) and run the fused
// epilogue: unscaling, the source update (1-lambda) B + lambda S, the residual
// max|S - S_prev|, the store of S and, in the source iteration, the
// relaxation Ibar <- 0.5 Ibar + 0.5 S written back in split form for the next
// step.  Every mbarrier wait is bounded (2 s of %globaltimer);
// a wait that gives up sets the context's device flag and the kernel drains
// and exits instead of hanging.
//
// Reference counterpart: d_GetS_MPI_Stream (cuda/cuda_kernel.cu:82-111) and
// its launch in CalculateIntScatteringAsyncMPIStream (cuda/cuda_solve.cu:89-111).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "rts_internal.h"

namespace {

constexpr int BM = 128;            // cells per tile (UMMA M, TMEM lanes)
constexpr int KS = 32;             // in-directions per stage (64 halves per row)
constexpr int MAX_BN = 256;        // out-directions per tile (UMMA N)
constexpr int A_BYTES = BM * 128;
constexpr int B_BYTES = MAX_BN * 128;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int DEFAULT_FLUSH = 1;   // stages (x32 in-directions) per hi*hi drain
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;  // 2 s per wait

enum { MODE_ITER = 0, MODE_ONESHOT = 1 };

// device flag codes
constexpr int FLAG_WAIT_PRODUCER = 1;
constexpr int FLAG_WAIT_MMA = 2;
constexpr int FLAG_WAIT_EPILOGUE = 4;
constexpr int FLAG_SCALE_OVERFLOW = 8;

// ------------------------------------------------------------------ PTX
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on a barrier phase; false (and the flag set) after the limit,
// or as soon as another CTA has given up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* flag, int code)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*(volatile int*)flag != 0) return false;
        if (global_ns() - t0 > WAIT_LIMIT_NS) {
            atomicOr(flag, code);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1 (tcgen05).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;            // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024u >> 4) << 32;  // stride byte offset
    d |= (uint64_t)1u << 46;            // version
    d |= (uint64_t)2u << 61;            // SWIZZLE_128B
    return d;
}

// ------------------------------------------------------------------ split helpers
template <bool kFp16>
struct Split;

template <>
struct Split<true> {
    static __device__ __forceinline__ void run(float x, uint16_t& hi, uint16_t& lo)
    {
        const __half h = __float2half_rn(x);
        const __half l = __float2half_rn(x - __half2float(h));
        hi = __half_as_ushort(h);
        lo = __half_as_ushort(l);
    }
    static __device__ __forceinline__ float join(uint16_t hi, uint16_t lo)
    {
        return __half2float(__ushort_as_half(hi)) + __half2float(__ushort_as_half(lo));
    }
};

template <>
struct Split<false> {
    static __device__ __forceinline__ void run(float x, uint16_t& hi, uint16_t& lo)
    {
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
        hi = __bfloat16_as_ushort(h);
        lo = __bfloat16_as_ushort(l);
    }
    static __device__ __forceinline__ float join(uint16_t hi, uint16_t lo)
    {
        return __bfloat162float(__ushort_as_bfloat16(hi)) + __bfloat162float(__ushort_as_bfloat16(lo));
    }
};

__device__ __forceinline__ uint32_t pack2(uint16_t a, uint16_t b) { return (uint32_t)a | ((uint32_t)b << 16); }

// offset (in halves) of the high part of in-direction j inside an interleaved row
__host__ __device__ __forceinline__ int64_t ilv_hi(int64_t j) { return (j >> 5) * 64 + (j & 31); }

// Power-of-two scale putting m into [2^13, 2^14): FP16 keeps 4x headroom.
__device__ __forceinline__ float pow2_scale(double m)
{
    if (!(m > 0.0) || !isfinite(m)) return 1.0f;
    const int e = ilogb(m);
    return ldexpf(1.0f, 13 - e);
}

// ------------------------------------------------------------------ prepasses
// W [Min][ldw] FP64 (column k = out-direction) -> Wc [mpad][2*kpad] split rows.
template <bool kFp16>
__global__ void split_w_kernel(const double* __restrict__ W, int Min, int Mout, int ldw, int kpad,
                               int mpad, uint16_t* __restrict__ Wc, float* __restrict__ cs,
                               float* __restrict__ cs_inv)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= mpad) return;
    uint16_t* row = Wc + (int64_t)k * 2 * kpad;
    if (k >= Mout) {
        for (int j = 0; j < 2 * kpad; ++j) row[j] = 0;
        cs[k] = 1.0f;
        cs_inv[k] = 1.0f;
        return;
    }
    float s = 1.0f;
    if (kFp16) {
        double m = 0.0;
        for (int j = 0; j < Min; ++j) m = fmax(m, fabs(W[(int64_t)j * ldw + k]));
        s = pow2_scale(m);
    }
    for (int j = 0; j < kpad; ++j) {
        uint16_t hi = 0, lo = 0;
        if (j < Min) Split<kFp16>::run((float)(W[(int64_t)j * ldw + k] * (double)s), hi, lo);
        row[ilv_hi(j)] = hi;
        row[ilv_hi(j) + 32] = lo;
    }
    cs[k] = s;
    cs_inv[k] = 1.0f / s;
}

// Row scale of every cell: max over directions of the face mean, and B.
__global__ void rowscale_kernel(const double* __restrict__ illum, int64_t N, int M,
                                const double* __restrict__ B, float* __restrict__ rs,
                                float* __restrict__ rs_inv, int64_t npad)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= npad) return;
    if (c >= N) {
        rs[c] = 1.0f;
        rs_inv[c] = 1.0f;
        return;
    }
    double m = B ? fabs(B[c]) : 0.0;
    for (int j = 0; j < M; ++j) {
        const double2* p = reinterpret_cast<const double2*>(illum + ((int64_t)j * N + c) * 4);
        const double2 a = __ldg(p), b = __ldg(p + 1);
        double I = 0.0;
        I += a.x;
        I += a.y;
        I += b.x;
        I += b.y;
        m = fmax(m, fabs(I / 4));
    }
    m *= 2.0;  // headroom for the relaxation S <= max(Ibar, B)
    const float s = pow2_scale(m);
    rs[c] = s;
    rs_inv[c] = 1.0f / s;
}

// Illum [M][N][4] FP64 -> A [npad][2*kpad] interleaved split rows (transpose
// through shared memory).  Tile: 32 in-directions x 64 cells, 256 threads.
template <bool kFp16>
__global__ void __launch_bounds__(256)
split_illum_kernel(const double* __restrict__ illum, int64_t N, int M, int kpad,
                   const float* __restrict__ rs, uint16_t* __restrict__ A)
{
    __shared__ float tile[64][33];
    const int j0 = blockIdx.y * 32;
    const int64_t c0 = (int64_t)blockIdx.x * 64;
    const int t = threadIdx.x;
    {
        const int cc = t & 63;
        const int64_t c = c0 + cc;
        const float s = (c < N && rs) ? rs[c] : 1.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int jj = (t >> 6) + 4 * q;
            const int j = j0 + jj;
            float v = 0.0f;
            if (c < N && j < M) {
                const double2* p = reinterpret_cast<const double2*>(illum + ((int64_t)j * N + c) * 4);
                const double2 a = __ldg(p), b = __ldg(p + 1);
                double I = 0.0;
                I += a.x;
                I += a.y;
                I += b.x;
                I += b.y;
                v = (float)((I / 4) * (double)s);
            }
            tile[cc][jj] = v;
        }
    }
    __syncthreads();
    // write: 64 rows x (hi 32 + lo 32) halves; each thread one row, 16 in-directions
    const int cc = t >> 2;
    const int part = t & 3;  // 0,1: hi of j 0-15 / 16-31; 2,3: lo of j 0-15 / 16-31
    const int64_t c = c0 + cc;
    if (c >= N) return;
    const int jbase = (part & 1) * 16;
    uint16_t out[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        uint16_t hi, lo;
        Split<kFp16>::run(tile[cc][jbase + i], hi, lo);
        out[i] = (part < 2) ? hi : lo;
    }
    uint16_t* dst = A + c * 2 * (int64_t)kpad + (int64_t)(j0 >> 5) * 64 + (part >= 2 ? 32 : 0) + jbase;
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    d4[0] = make_uint4(pack2(out[0], out[1]), pack2(out[2], out[3]), pack2(out[4], out[5]), pack2(out[6], out[7]));
    d4[1] = make_uint4(pack2(out[8], out[9]), pack2(out[10], out[11]), pack2(out[12], out[13]),
                       pack2(out[14], out[15]));
}

// Ibar [M][N] FP64 from the split rows (for inspection).
template <bool kFp16>
__global__ void join_illum_kernel(const uint16_t* __restrict__ A, int64_t N, int M, int kpad,
                                  const float* __restrict__ rs_inv, double* __restrict__ out)
{
    const int64_t total = (int64_t)M * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = i / N, c = i % N;
        const uint16_t* row = A + c * 2 * (int64_t)kpad;
        const float x = Split<kFp16>::join(row[ilv_hi(j)], row[ilv_hi(j) + 32]);
        out[i] = (double)x * (double)(rs_inv ? rs_inv[c] : 1.0f);
    }
}

__global__ void s32_to_f64_kernel(const float* __restrict__ s, double* __restrict__ d, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (double)s[i];
}

// ------------------------------------------------------------------ GEMM
#include "rts_split_gemm.cuh"

// ------------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 get_encode(rts_ctx* ctx)
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (fn) return fn;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
        cudaGetLastError();
        rts_fail(ctx, RTS_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        return nullptr;
    }
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return fn;
}

// 2-D map over an interleaved split operand [rows][2*kpad] (16-bit), box
// 64 halves x box_rows, 128-byte swizzle.
int make_map(rts_ctx* ctx, CUtensorMap* map, const void* base, int64_t rows, int64_t kpad, int box_rows)
{
    auto enc = get_encode(ctx);
    if (!enc) return RTS_ERR_CUDA;
    cuuint64_t dims[2] = {(cuuint64_t)(2 * kpad), (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(2 * kpad * 2)};
    cuuint32_t box[2] = {64u, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1u, 1u};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return rts_fail(ctx, RTS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) for %lld x %lld", (int)r,
                        (long long)rows, (long long)(2 * kpad));
    return RTS_OK;
}

uint32_t make_idesc(bool fp16, int bn)
{
    const uint32_t ab = fp16 ? 0u : 1u;  // 0 = F16, 1 = BF16
    return (1u << 4)                     // D = F32
           | (ab << 7) | (ab << 10)      // A, B formats
           | ((uint32_t)(bn >> 3) << 17) // N >> 3
           | ((uint32_t)(BM >> 4) << 24);  // M >> 4
}

int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

int choose_bn(int64_t mout)
{
    if (mout >= 256) return 256;
    return (int)round_up(mout, 16);
}

CUtensorMap* map_a(rts_ctx* ctx, int i) { return reinterpret_cast<CUtensorMap*>(ctx->split.maps[i]); }
CUtensorMap* map_w(rts_ctx* ctx) { return reinterpret_cast<CUtensorMap*>(ctx->split.maps[2]); }

template <bool kFp16, int kMode>
int launch_gemm(rts_ctx* ctx, const CUtensorMap& mA, const CUtensorMap& mB, const GemmArgs& a,
                int64_t m_tiles, cudaStream_t st)
{
    auto kern = split_gemm_kernel<kFp16, kMode>;
    RTS_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GEMM_SMEM2));
    const int64_t grid = m_tiles * a.n_tiles;
    RTS_REQUIRE(ctx, grid < (1ll << 31), RTS_ERR_UNSUPPORTED, "tensor-path grid too large");
    rts_timing_begin(ctx, st);
    kern<<<(unsigned)grid, GEMM_THREADS2, GEMM_SMEM2, st>>>(mA, mB, a);
    rts_timing_end(ctx, st);
    RTS_CHECK_LAUNCH(ctx, "split_gemm_kernel");
    ctx->launches++;
    return RTS_OK;
}

int grid_for(rts_ctx* ctx, int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)ctx->num_sms * 16;
    return (int)(b > cap ? cap : (b < 1 ? 1 : b));
}

// Allocate (or reuse) the split buffers for an M_in x M_out problem on N cells.
int ensure_buffers(rts_ctx* ctx, int precision, bool iterative)
{
    rts_split_state& sp = ctx->split;
    const int64_t Min = ctx->M, Mout = ctx->local(), N = ctx->N;
    const int64_t kpad = round_up(Min, KS);
    const int bn = choose_bn(Mout);
    const int64_t mpad = round_up(Mout, bn);
    const int64_t npad = round_up(N, BM);
    const bool same = sp.precision >= 0 && sp.kpad == kpad && sp.mpad == mpad && sp.npad == npad &&
                      (!iterative || (sp.i_hi[1] && sp.s32));
    if (!same) {
        rts_split_free(ctx);
        void* p;
        int st;
#define SPLIT_ALLOC(dst, bytes, name)                                  \
    if ((st = rts_dmalloc(ctx, &p, (bytes), name)) != RTS_OK) {        \
        rts_split_free(ctx);                                           \
        return st;                                                     \
    }                                                                  \
    dst = (decltype(dst))p;
        SPLIT_ALLOC(sp.w_hi, (size_t)(mpad * 2 * kpad * 2), "split W");
        SPLIT_ALLOC(sp.w_colscale, (size_t)(mpad * 4 * 2), "W column scales");
        SPLIT_ALLOC(sp.i_hi[0], (size_t)(npad * 2 * kpad * 2), "split Ibar");
        SPLIT_ALLOC(sp.i_rowscale[0], (size_t)(npad * 4 * 2), "Ibar row scales");
        if (iterative) {
            SPLIT_ALLOC(sp.i_hi[1], (size_t)(npad * 2 * kpad * 2), "split Ibar (next)");
            SPLIT_ALLOC(sp.s32, (size_t)(Mout * N * 4), "FP32 scattering");
        }
#undef SPLIT_ALLOC
        sp.kpad = kpad;
        sp.mpad = mpad;
        sp.npad = npad;
        RTS_CUDA_TRY(ctx, cudaMemset(sp.i_hi[0], 0, (size_t)(npad * 2 * kpad * 2)));
        if (sp.i_hi[1]) RTS_CUDA_TRY(ctx, cudaMemset(sp.i_hi[1], 0, (size_t)(npad * 2 * kpad * 2)));
        int rc = make_map(ctx, map_w(ctx), sp.w_hi, mpad, kpad, bn);
        if (rc == RTS_OK) rc = make_map(ctx, map_a(ctx, 0), sp.i_hi[0], npad, kpad, BM);
        if (rc == RTS_OK && sp.i_hi[1]) rc = make_map(ctx, map_a(ctx, 1), sp.i_hi[1], npad, kpad, BM);
        if (rc != RTS_OK) {
            rts_split_free(ctx);
            return rc;
        }
        sp.bn = bn;
    }
    sp.precision = precision;
    return RTS_OK;
}

float* rowscale_inv(rts_ctx* ctx) { return ctx->split.i_rowscale[0] + ctx->split.npad; }
float* colscale_inv(rts_ctx* ctx) { return ctx->split.w_colscale + ctx->split.mpad; }

// W split + Ibar split from the device Illum (faces) into buffer 0.
int prepare_operands(rts_ctx* ctx, bool fp16, const double* B, cudaStream_t st)
{
    rts_split_state& sp = ctx->split;
    const int Min = (int)ctx->M, Mout = (int)ctx->local();
    const int kpad = (int)sp.kpad, mpad = (int)sp.mpad;
    if (fp16)
        split_w_kernel<true><<<(mpad + 127) / 128, 128, 0, st>>>(ctx->d_W, Min, Mout, Mout, kpad, mpad,
                                                                 (uint16_t*)sp.w_hi, sp.w_colscale,
                                                                 colscale_inv(ctx));
    else
        split_w_kernel<false><<<(mpad + 127) / 128, 128, 0, st>>>(ctx->d_W, Min, Mout, Mout, kpad, mpad,
                                                                  (uint16_t*)sp.w_hi, sp.w_colscale,
                                                                  colscale_inv(ctx));
    RTS_CHECK_LAUNCH(ctx, "split_w_kernel");
    ctx->launches++;
    float* rs = sp.i_rowscale[0];
    if (fp16) {
        rowscale_kernel<<<(unsigned)((sp.npad + 127) / 128), 128, 0, st>>>(ctx->d_illum, ctx->N, Min, B, rs,
                                                                           rowscale_inv(ctx), sp.npad);
        RTS_CHECK_LAUNCH(ctx, "rowscale_kernel");
        ctx->launches++;
    }
    dim3 grid((unsigned)((ctx->N + 63) / 64), (unsigned)(kpad / 32));
    if (fp16)
        split_illum_kernel<true><<<grid, 256, 0, st>>>(ctx->d_illum, ctx->N, Min, kpad, rs, (uint16_t*)sp.i_hi[0]);
    else
        split_illum_kernel<false><<<grid, 256, 0, st>>>(ctx->d_illum, ctx->N, Min, kpad, nullptr,
                                                        (uint16_t*)sp.i_hi[0]);
    RTS_CHECK_LAUNCH(ctx, "split_illum_kernel");
    ctx->launches++;
    return RTS_OK;
}

GemmArgs base_args(rts_ctx* ctx, bool fp16)
{
    rts_split_state& sp = ctx->split;
    GemmArgs a;
    memset(&a, 0, sizeof(a));
    a.N = ctx->N;
    a.Mout = (int)ctx->local();
    a.kpad = (int)sp.kpad;
    a.kblocks = (int)(sp.kpad / KS);
    a.bn = sp.bn;
    a.n_tiles = (int)(sp.mpad / a.bn);
    a.idesc = make_idesc(fp16, a.bn);
    a.flush = ctx->split_flush > 0 ? ctx->split_flush : DEFAULT_FLUSH;
    a.rs = fp16 ? sp.i_rowscale[0] : nullptr;
    a.rs_inv = fp16 ? rowscale_inv(ctx) : nullptr;
    a.cs_inv = fp16 ? colscale_inv(ctx) : nullptr;
    a.flag = ctx->d_flag;
    a.resid = ctx->resid_target;
    return a;
}

}  // namespace

int rts_split_setup(rts_ctx* ctx, int precision)
{
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED,
                "the tensor-core path needs a Blackwell (sm_10x) device, found sm_%d%d", ctx->cc_major,
                ctx->cc_minor);
    const bool fp16 = precision == RTS_PREC_FP16X3;
    int rc = ensure_buffers(ctx, precision, true);
    if (rc != RTS_OK) return rc;
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), st));
    rc = prepare_operands(ctx, fp16, ctx->d_B, st);
    if (rc != RTS_OK) return rc;
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(ctx->split.s32, 0, (size_t)(ctx->local() * ctx->N * 4), st));
    ctx->split.cur = 0;
    // the second Ibar buffer shares the row scales of the first
    ctx->split.i_rowscale[1] = ctx->split.i_rowscale[0];
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return RTS_OK;
}

int rts_split_step(rts_ctx* ctx, bool relax, cudaStream_t st)
{
    rts_split_state& sp = ctx->split;
    const bool fp16 = sp.precision == RTS_PREC_FP16X3;
    RTS_REQUIRE(ctx, relax == false || ctx->local() == ctx->M, RTS_ERR_UNSUPPORTED,
                "relaxation needs all out-directions local");
    GemmArgs a = base_args(ctx, fp16);
    a.B = ctx->d_B;
    a.lam = (float)ctx->solve_lambda;
    a.S32 = sp.s32;
    a.a_cur = (const uint16_t*)sp.i_hi[sp.cur];
    a.a_next = (uint16_t*)sp.i_hi[sp.cur ^ 1];
    a.relax = relax ? 1 : 0;
    a.residual = 1;
    const int64_t m_tiles = sp.npad / BM;
    int rc = fp16 ? launch_gemm<true, MODE_ITER>(ctx, *map_a(ctx, sp.cur), *map_w(ctx), a, m_tiles, st)
                  : launch_gemm<false, MODE_ITER>(ctx, *map_a(ctx, sp.cur), *map_w(ctx), a, m_tiles, st);
    if (rc != RTS_OK) return rc;
    if (relax) sp.cur ^= 1;
    return RTS_OK;
}

int rts_split_oneshot(rts_ctx* ctx, int precision, const double* B, double lambda, cudaStream_t st)
{
    RTS_REQUIRE(ctx, ctx->cc_major == 10, RTS_ERR_UNSUPPORTED,
                "the tensor-core path needs a Blackwell (sm_10x) device");
    const bool fp16 = precision == RTS_PREC_FP16X3;
    const bool had_iter = ctx->split.s32 != nullptr;
    int rc = ensure_buffers(ctx, precision, had_iter);
    if (rc != RTS_OK) return rc;
    ctx->solve_ready = false;  // buffer 0 is overwritten
    rc = prepare_operands(ctx, fp16, B, st);
    if (rc != RTS_OK) return rc;
    GemmArgs a = base_args(ctx, fp16);
    a.B = B;
    a.lam = (float)lambda;
    a.S64 = ctx->d_S;
    a.a_cur = (const uint16_t*)ctx->split.i_hi[0];
    const int64_t m_tiles = ctx->split.npad / BM;
    return fp16 ? launch_gemm<true, MODE_ONESHOT>(ctx, *map_a(ctx, 0), *map_w(ctx), a, m_tiles, st)
                : launch_gemm<false, MODE_ONESHOT>(ctx, *map_a(ctx, 0), *map_w(ctx), a, m_tiles, st);
}

int rts_split_read(rts_ctx* ctx, double* S_host)
{
    rts_split_state& sp = ctx->split;
    RTS_REQUIRE(ctx, sp.s32, RTS_ERR_BAD_STATE, "no tensor-path source iteration set up");
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    const int64_t n = ctx->local() * ctx->N;
    // d_S is free scratch on the tensor path
    s32_to_f64_kernel<<<grid_for(ctx, n, 256), 256, 0, st>>>(sp.s32, ctx->d_S, n);
    RTS_CHECK_LAUNCH(ctx, "s32_to_f64_kernel");
    ctx->launches++;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(S_host, ctx->d_S, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    int flag = 0;
    RTS_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag)
        return rts_fail(ctx, RTS_ERR_DEVICE_WAIT, "tensor-path kernel reported device flag %d", flag);
    return RTS_OK;
}

int rts_split_read_ibar(rts_ctx* ctx, double* ibar_host)
{
    rts_split_state& sp = ctx->split;
    RTS_REQUIRE(ctx, sp.i_hi[0], RTS_ERR_BAD_STATE, "no tensor-path operands set up");
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    const int64_t n = ctx->M * ctx->N;
    const bool fp16 = sp.precision == RTS_PREC_FP16X3;
    double* tmp = nullptr;
    int rc = rts_dmalloc(ctx, (void**)&tmp, (size_t)n * 8, "Ibar readback");
    if (rc != RTS_OK) return rc;
    const uint16_t* A = (const uint16_t*)sp.i_hi[sp.cur];
    if (fp16)
        join_illum_kernel<true><<<grid_for(ctx, n, 256), 256, 0, st>>>(A, ctx->N, (int)ctx->M, (int)sp.kpad,
                                                                      rowscale_inv(ctx), tmp);
    else
        join_illum_kernel<false><<<grid_for(ctx, n, 256), 256, 0, st>>>(A, ctx->N, (int)ctx->M, (int)sp.kpad,
                                                                       nullptr, tmp);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(ibar_host, tmp, (size_t)n * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    rts_dfree(ctx, tmp, (size_t)n * 8);
    if (e != cudaSuccess) return rts_fail(ctx, RTS_ERR_CUDA, "Ibar readback failed: %s", cudaGetErrorString(e));
    ctx->launches++;
    return RTS_OK;
}

void rts_split_free(rts_ctx* ctx)
{
    rts_split_state& sp = ctx->split;
    const size_t a_bytes = (size_t)(sp.npad * 2 * sp.kpad * 2);
    rts_dfree(ctx, sp.w_hi, (size_t)(sp.mpad * 2 * sp.kpad * 2));
    rts_dfree(ctx, sp.w_colscale, (size_t)(sp.mpad * 4 * 2));
    rts_dfree(ctx, sp.i_hi[0], a_bytes);
    rts_dfree(ctx, sp.i_hi[1], a_bytes);
    rts_dfree(ctx, sp.i_rowscale[0], (size_t)(sp.npad * 4 * 2));
    rts_dfree(ctx, sp.s32, (size_t)(ctx->local() * ctx->N * 4));
    sp = rts_split_state();
}
