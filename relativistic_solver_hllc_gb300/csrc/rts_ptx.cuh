// rts_ptx.cuh -- inline-PTX building blocks of the tcgen05 kernels (sm_103a):
// mbarriers with bounded waits, TMA tile loads, TMEM allocation / load /
// store, tcgen05.mma (kind::f16) and its commit, shared-memory matrix
// descriptors, and the FP16 / BF16 hi-lo split.  Header-only; every
// function is internal to the including translation unit.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>

namespace rts_ptx {

constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;  // 2 s per wait

// device flag codes (bitwise OR into the context's flag word)
constexpr int FLAG_WAIT_PRODUCER = 1;
constexpr int FLAG_WAIT_MMA = 2;
constexpr int FLAG_WAIT_EPILOGUE = 4;
constexpr int FLAG_SCALE_OVERFLOW = 8;
constexpr int FLAG_WAIT_STORE = 16;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

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
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
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

// Bounded wait on a barrier phase.  Returns false (flag set) after
// WAIT_LIMIT_NS, or as soon as another CTA has set the flag; the flag word
// is polled only every 256 attempts so a healthy wait costs no global loads.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* flag, int code)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t n = 1;; ++n) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((n & 255u) == 0) {
            if (*(volatile int*)flag != 0) return false;
            if (global_ns() - t0 > WAIT_LIMIT_NS) {
                atomicOr(flag, code);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void* map, int x, int y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Bulk tensor store of a shared-memory box to global memory (bulk-group
// completion), its commit, and the waits: until the sources have been read
// (the shared memory may be reused) or until the writes are done.
__device__ __forceinline__ void tma_store_2d(const void* map, int x, int y, uint32_t src)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(src)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// Orders this thread's generic-proxy shared-memory writes before later
// async-proxy (TMA) reads of the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// tcgen05.mma kind::tf32 (K = 8 per instruction: 32 bytes of each row, the
// same bytes as one kind::f16 step).
__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns (one row per thread); load and
// wait in one asm statement so no use can be scheduled before the wait.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 32 consecutive 32-bit columns, load and wait in one asm
// statement (tcgen05.ld destinations are not scoreboarded: no use may be
// scheduled before the wait).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 8 consecutive 32-bit columns, load and wait in one statement.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// 16-byte asynchronous global -> shared copy (cp.async, L2 only).
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void prefetch_l2(const void* p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
        "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
        "r"(__float_as_uint(v[15]))
        : "memory");
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1 (tcgen05).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;            // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024u >> 4) << 32;  // stride byte offset
    d |= (uint64_t)1u << 46;            // descriptor version
    d |= (uint64_t)2u << 61;            // SWIZZLE_128B
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D = F32, A and B of the
// same 16-bit type (0 = F16, 1 = BF16), both K-major, M = 128, N = bn.
__host__ __device__ __forceinline__ uint32_t idesc_f16(bool fp16, int m, int n)
{
    const uint32_t ab = fp16 ? 0u : 1u;
    return (1u << 4) | (ab << 7) | (ab << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Instruction descriptor for split mode 0 (BF16, kind::f16), 1 (FP16,
// kind::f16) or 2 (TF32, kind::tf32: A and B format 2).  D = F32, K-major.
__host__ __device__ __forceinline__ uint32_t idesc_split(int mode, int m, int n)
{
    const uint32_t ab = mode == 1 ? 0u : mode == 0 ? 1u : 2u;
    return (1u << 4) | (ab << 7) | (ab << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// ------------------------------------------------------------- hi / lo split
__device__ __forceinline__ void split_f16(float x, uint16_t& hi, uint16_t& lo)
{
    const __half h = __float2half_rn(x);
    const __half l = __float2half_rn(x - __half2float(h));
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(l);
}
__device__ __forceinline__ float join_f16(uint16_t hi, uint16_t lo)
{
    return __half2float(__ushort_as_half(hi)) + __half2float(__ushort_as_half(lo));
}
__device__ __forceinline__ void split_bf16(float x, uint16_t& hi, uint16_t& lo)
{
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    hi = __bfloat16_as_ushort(h);
    lo = __bfloat16_as_ushort(l);
}
__device__ __forceinline__ float join_bf16(uint16_t hi, uint16_t lo)
{
    return __bfloat162float(__ushort_as_bfloat16(hi)) + __bfloat162float(__ushort_as_bfloat16(lo));
}
__device__ __forceinline__ void split_any(bool fp16, float x, uint16_t& hi, uint16_t& lo)
{
    if (fp16)
        split_f16(x, hi, lo);
    else
        split_bf16(x, hi, lo);
}
__device__ __forceinline__ float join_any(bool fp16, uint16_t hi, uint16_t lo)
{
    return fp16 ? join_f16(hi, lo) : join_bf16(hi, lo);
}

__host__ __device__ __forceinline__ uint32_t pack2(uint16_t a, uint16_t b) { return (uint32_t)a | ((uint32_t)b << 16); }

// Two values at once (first in the low half), bit-identical to split_any /
// join_any on each value.
__device__ __forceinline__ void split2_any(bool fp16, float x0, float x1, uint32_t& hi2, uint32_t& lo2)
{
    if (fp16) {
        const __half2 h = __floats2half2_rn(x0, x1);
        const float2 b = __half22float2(h);
        const __half2 l = __floats2half2_rn(x0 - b.x, x1 - b.y);
        hi2 = *reinterpret_cast<const uint32_t*>(&h);
        lo2 = *reinterpret_cast<const uint32_t*>(&l);
    } else {
        const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
        const float2 b = __bfloat1622float2(h);
        const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - b.x, x1 - b.y);
        hi2 = *reinterpret_cast<const uint32_t*>(&h);
        lo2 = *reinterpret_cast<const uint32_t*>(&l);
    }
}
__device__ __forceinline__ float2 join2_any(bool fp16, uint32_t hi2, uint32_t lo2)
{
    float2 h, l;
    if (fp16) {
        h = __half22float2(*reinterpret_cast<const __half2*>(&hi2));
        l = __half22float2(*reinterpret_cast<const __half2*>(&lo2));
    } else {
        h = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hi2));
        l = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&lo2));
    }
    return make_float2(h.x + l.x, h.y + l.y);
}

// offset (in halves) of the high part of in-direction j inside an interleaved
// split row: per 32 in-directions, 32 high halves then 32 low halves
__host__ __device__ __forceinline__ int64_t ilv_hi(int64_t j) { return (j >> 5) * 64 + (j & 31); }

// ------------------------------------------------------------ TF32 hi / lo split
// TF32 keeps FP32's 8-bit exponent and 10 explicit mantissa bits.  x = hi +
// lo with hi = x rounded to TF32 (round to nearest, ties away) and lo = the
// rounded remainder, so hi + lo carries 22 significant bits; both are stored
// as FP32 bit patterns whose low 13 bits are zero (the tensor core reads the
// upper 19 bits).  Rows of the split operands hold, for each group of 16
// in-directions, 16 high parts then 16 low parts (128 bytes): the same bytes
// per K-slice as the 16-bit split, at half the in-directions.
__device__ __forceinline__ float tf32_round(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo)
{
    hi = tf32_round(x);
    lo = tf32_round(x - hi);
}

// position of in-direction j's high part in a TF32 split row (FP32 units)
__host__ __device__ __forceinline__ int64_t ilv_hi_tf32(int64_t j) { return (j >> 4) * 32 + (j & 15); }

}  // namespace rts_ptx
