// rts_split_gemm.cuh -- the tcgen05 contraction kernel of the split-precision
// path (included by rts_split.cu; relies on its PTX helpers and constants).
//
// Accuracy design.  The tensor core adds every MMA result into its FP32
// accumulator with truncation, so a long accumulation drifts low by about a
// quarter of an FP32 ulp per MMA.  Two measures keep the drift below 3e-7:
//   * the hi*hi product and the two cross products (hi*lo, lo*hi, 2^-11 or
//     2^-8 smaller) accumulate in separate TMEM accumulators, so the many
//     cross MMAs truncate at the small accumulator's ulp;
//   * the hi*hi accumulator is drained every FLUSH stages (FLUSH*32 in-
//     directions) into FP32 registers of the epilogue warps, where partial
//     sums are added with round-to-nearest; the MMA warp issues the next
//     stage's cross products while the drain runs.
//
// Roles (320 threads): warp 0 TMA producer, warp 1 TMEM owner + MMA issuer,
// warps 2..9 epilogue (two warps per TMEM lane quarter, one per half of the
// 256 accumulator columns; 128 running sums per thread).  TMEM: columns
// [0,256) hi*hi, [256,512) cross terms -- the whole TMEM, one CTA per SM.

constexpr int EPI_WARPS = 8;
constexpr int GEMM_THREADS2 = 64 + 32 * EPI_WARPS;
constexpr uint32_t TMEM_COLS2 = 512;
constexpr int STAGES2 = 4;
constexpr size_t GEMM_SMEM2 = (size_t)STAGES2 * STAGE_BYTES + 1024 + 256;

struct GemmArgs {
    int64_t N;        // cells
    int Mout;         // valid out-directions (columns of D)
    int kblocks;      // kpad / 32
    int kpad;
    int bn;           // columns per tile
    int n_tiles;
    int flush;        // stages per hi*hi drain
    uint32_t idesc;
    const float* rs_inv;  // [npad] or null (BF16)
    const float* rs;
    const float* cs_inv;  // [mpad] or null
    const double* B;      // [N] or null (no update)
    float lam;
    float* S32;           // MODE_ITER: [Mout][N]
    double* S64;          // MODE_ONESHOT: [Mout][N]
    const uint16_t* a_cur;
    uint16_t* a_next;     // relaxation target (MODE_ITER, relax)
    int relax;
    int residual;
    unsigned long long* resid;
    int* flag;
};

template <bool kFp16, int kMode>
__global__ void __launch_bounds__(GEMM_THREADS2, 1)
split_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const GemmArgs args)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES2 * STAGE_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES2 + 3);
    const uint32_t smem_base = smem_u32(smem);
    const uint32_t bar_base = smem_u32(bars);
    auto full_bar = [&](int s) { return bar_base + 8u * s; };
    auto empty_bar = [&](int s) { return bar_base + 8u * (STAGES2 + s); };
    const uint32_t hh_full_bar = bar_base + 8u * (2 * STAGES2);
    const uint32_t hh_empty_bar = hh_full_bar + 8u;
    const uint32_t tmem_full_bar = hh_full_bar + 16u;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_tile = blockIdx.x % args.n_tiles;
    const int64_t m_tile = blockIdx.x / args.n_tiles;
    const int bn = args.bn;
    const int nkb = args.kblocks;
    const int flush = args.flush;
    const int nchunks = (nkb + flush - 1) / flush;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES2; ++s) {
            mbar_init(full_bar(s), 1);
            mbar_init(empty_bar(s), 1);
        }
        mbar_init(hh_full_bar, 1);
        mbar_init(hh_empty_bar, EPI_WARPS);
        mbar_init(tmem_full_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(smem_u32(tmem_slot), TMEM_COLS2);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t tmem_hh = tmem, tmem_x = tmem + 256u;
    const bool live = *(volatile int*)args.flag == 0;

    if (warp == 0) {
        if (lane == 0 && live) {
            // ---------------- TMA producer
            const uint32_t tx = (uint32_t)(A_BYTES + bn * 128);
            int kb = 0;
            for (; kb < nkb; ++kb) {
                const int s = kb % STAGES2;
                if (kb >= STAGES2 &&
                    !mbar_wait(empty_bar(s), ((kb / STAGES2) - 1) & 1, args.flag, FLAG_WAIT_PRODUCER))
                    break;
                mbar_expect_tx(full_bar(s), tx);
                const uint32_t sa = smem_base + s * STAGE_BYTES;
                tma_load_2d(sa, &tmA, kb * 64, (int)(m_tile * BM), full_bar(s));
                tma_load_2d(sa + A_BYTES, &tmB, kb * 64, n_tile * bn, full_bar(s));
            }
            for (int i = (kb > STAGES2 ? kb - STAGES2 : 0); i < kb; ++i)
                mbar_wait(full_bar(i % STAGES2), (i / STAGES2) & 1, args.flag, FLAG_WAIT_PRODUCER);
        }
    } else if (warp == 1) {
        if (lane == 0 && live) {
            // ---------------- MMA issuer
            bool ok = true;
            for (int kb = 0; kb < nkb && ok; ++kb) {
                const int s = kb % STAGES2;
                const int chunk = kb / flush;
                const bool chunk_first = (kb % flush) == 0;
                const bool chunk_last = (kb % flush) == flush - 1 || kb == nkb - 1;
                if (!mbar_wait(full_bar(s), (kb / STAGES2) & 1, args.flag, FLAG_WAIT_MMA)) break;
                tc_fence_after();
                const uint32_t sa = smem_base + s * STAGE_BYTES;
                const uint64_t ad = smem_desc_sw128(sa);
                const uint64_t bd = smem_desc_sw128(sa + A_BYTES);
                const uint64_t hi0 = 0, hi1 = 32 >> 4, lo0 = 64 >> 4, lo1 = 96 >> 4;
                // cross products first: they overlap the drain of the previous chunk
                umma_f16(tmem_x, ad + hi0, bd + lo0, args.idesc, kb != 0 ? 1u : 0u);
                umma_f16(tmem_x, ad + lo0, bd + hi0, args.idesc, 1u);
                umma_f16(tmem_x, ad + hi1, bd + lo1, args.idesc, 1u);
                umma_f16(tmem_x, ad + lo1, bd + hi1, args.idesc, 1u);
                if (chunk_first && chunk > 0) {
                    // the epilogue must have drained the previous hi*hi partial
                    if (!mbar_wait(hh_empty_bar, (chunk - 1) & 1, args.flag, FLAG_WAIT_MMA)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                }
                umma_f16(tmem_hh, ad + hi0, bd + hi0, args.idesc, chunk_first ? 0u : 1u);
                umma_f16(tmem_hh, ad + hi1, bd + hi1, args.idesc, 1u);
                umma_commit(empty_bar(s));
                if (chunk_last && kb != nkb - 1) umma_commit(hh_full_bar);
            }
            umma_commit(tmem_full_bar);  // also after a failed wait: drains issued MMAs
        }
    } else {
        // ---------------- epilogue
        const int ew = warp - 2;
        const int q = warp & 3;          // TMEM lane quarter
        const int h = ew >> 2;           // column half
        const int64_t c = m_tile * BM + q * 32 + lane;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        const int col0 = h * 128;
        const bool active = col0 < bn;   // warp-uniform
        float run[128];
#pragma unroll
        for (int i = 0; i < 128; ++i) run[i] = 0.0f;
        bool ok = live;
        for (int chunk = 0; chunk + 1 < nchunks && ok; ++chunk) {
            bool got = true;
            if (lane == 0) got = mbar_wait(hh_full_bar, chunk & 1, args.flag, FLAG_WAIT_EPILOGUE);
            ok = __shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0;
            if (!ok) break;
            tc_fence_after();
            if (active) {
#pragma unroll
                for (int g = 0; g < 8; ++g) {
                    float v[16];
                    tmem_ld16(tmem_hh + lane_off + (uint32_t)(col0 + 16 * g), v);
#pragma unroll
                    for (int i = 0; i < 16; ++i) run[16 * g + i] += v[i];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(hh_empty_bar) : "memory");
        }
        bool got = true;
        if (lane == 0) got = mbar_wait(tmem_full_bar, 0, args.flag, FLAG_WAIT_EPILOGUE);
        ok = ok && (__shfl_sync(0xffffffffu, got ? 1 : 0, 0) != 0);
        tc_fence_after();
        if (ok && active) {
            const bool in_row = c < args.N;
            const float rinv = (kFp16 && in_row) ? args.rs_inv[c] : 1.0f;
            const float rsc = (kFp16 && in_row) ? args.rs[c] : 1.0f;
            const float bterm = (args.B && in_row) ? (float)((1.0 - (double)args.lam) * args.B[c]) : 0.0f;
            const float lam = args.B ? args.lam : 1.0f;
            float rmax = 0.0f;
            bool overflow = false;
#pragma unroll
            for (int g = 0; g < 8; ++g) {
                float vh[16], vx[16];
                tmem_ld16(tmem_hh + lane_off + (uint32_t)(col0 + 16 * g), vh);
                tmem_ld16(tmem_x + lane_off + (uint32_t)(col0 + 16 * g), vx);
                const int k0 = n_tile * bn + col0 + 16 * g;
                if (!in_row || k0 >= args.Mout || col0 + 16 * g >= bn) continue;
                float v[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = (run[16 * g + i] + vh[i]) + vx[i];
                if (kMode == MODE_ITER) {
                    uint16_t nh[16], nl[16];
                    uint4 ch_hi[2], ch_lo[2];
                    const bool do_relax = args.relax && k0 < args.kpad;
                    if (do_relax) {
                        const uint4* src = reinterpret_cast<const uint4*>(args.a_cur + c * 2 * (int64_t)args.kpad + ilv_hi(k0));
                        ch_hi[0] = src[0];
                        ch_hi[1] = src[1];
                        ch_lo[0] = src[4];
                        ch_lo[1] = src[5];
                    }
                    const uint16_t* ph = reinterpret_cast<const uint16_t*>(ch_hi);
                    const uint16_t* pl = reinterpret_cast<const uint16_t*>(ch_lo);
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int k = k0 + i;
                        float xnext = 0.0f;
                        if (k < args.Mout) {
                            const float cinv = kFp16 ? __ldg(args.cs_inv + k) : 1.0f;
                            const float sint = v[i] * rinv * cinv;
                            const float snew = bterm + lam * sint;
                            float* dst = args.S32 + (int64_t)k * args.N + c;
                            if (args.residual) rmax = fmaxf(rmax, fabsf(snew - *dst));
                            *dst = snew;
                            if (do_relax) xnext = 0.5f * Split<kFp16>::join(ph[i], pl[i]) + 0.5f * (snew * rsc);
                        }
                        if (do_relax) {
                            if (kFp16 && fabsf(xnext) > 60000.0f) overflow = true;
                            Split<kFp16>::run(xnext, nh[i], nl[i]);
                        }
                    }
                    if (do_relax) {
                        uint4* dst = reinterpret_cast<uint4*>(args.a_next + c * 2 * (int64_t)args.kpad + ilv_hi(k0));
                        const uint32_t* h32 = reinterpret_cast<const uint32_t*>(nh);
                        const uint32_t* l32 = reinterpret_cast<const uint32_t*>(nl);
                        dst[0] = make_uint4(h32[0], h32[1], h32[2], h32[3]);
                        dst[1] = make_uint4(h32[4], h32[5], h32[6], h32[7]);
                        dst[4] = make_uint4(l32[0], l32[1], l32[2], l32[3]);
                        dst[5] = make_uint4(l32[4], l32[5], l32[6], l32[7]);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int k = k0 + i;
                        if (k < args.Mout) {
                            const float cinv = kFp16 ? __ldg(args.cs_inv + k) : 1.0f;
                            const float sint = v[i] * rinv * cinv;
                            args.S64[(int64_t)k * args.N + c] = (double)(bterm + lam * sint);
                        }
                    }
                }
            }
            if (overflow) atomicOr(args.flag, FLAG_SCALE_OVERFLOW);
            if (kMode == MODE_ITER && args.residual) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
                if (lane == 0 && rmax > 0.0f)
                    atomicMax(args.resid, (unsigned long long)__double_as_longlong((double)rmax));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, TMEM_COLS2);
    }
}
