// rts_group_kernel.cuh -- persistent, grouped tcgen05 contraction of the
// split-precision scattering integral (included by rts_group.cu).
//
// One launch runs one source-iteration step of every problem of a batch: the
// tiles of all problems (128 cells x up to 128 out-directions each; problems
// of different cell and direction counts, phase kernels and precisions) form
// one list that persistent CTAs walk with a fixed stride.
//
// Two CTAs run on every SM.  Measured on GB300, one CTA issuing
// tcgen05.mma back to back gets one instruction through every ~280 cycles
// whatever N is, while the SM's tensor core sustains several such streams;
// two resident CTAs (each with its own issuing thread) double the tensor
// throughput of the SM, and one CTA's epilogue overlaps the other's main loop.
//
// Warp roles (192 threads per CTA):
//   warp 0      TMA producer: A (split Ibar rows) and B (split W rows)
//               K-slices into a 3-stage shared-memory ring;
//   warp 1      TMEM owner (256 columns) and single-thread MMA issuer;
//   warps 2..5  epilogue: drain the accumulator of every `flush` K-slices into
//               FP32 registers (round-to-nearest adds; the tensor core
//               truncates each accumulate), then for the finished tile run the
//               fused epilogue (unscaling, source update, residual, S store,
//               relaxation of Ibar in split form).
// TMEM: two accumulators of 128 columns used alternately per chunk of
// `flush` K-slices, so the MMAs of one chunk run while the previous chunk is
// drained.  Within a chunk the cross products hi*lo and lo*hi (2^-11 or 2^-8
// of the result) are issued first, while the accumulator is still small, and
// the two hi*hi products last: the truncation then costs about one FP32 ulp of
// the chunk sum per hi*hi MMA, as with separate accumulators.
//
// Every mbarrier wait is bounded (rts_ptx::mbar_wait); a wait that gives up
// sets the device flag, every role stops at its next wait, and the kernel
// drains and exits.

constexpr int G_BM = 128;
constexpr int G_BN = 128;
constexpr int G_STAGES = 3;
constexpr int G_A_BYTES = G_BM * 128;
constexpr int G_B_BYTES = G_BN * 128;
constexpr int G_STAGE_BYTES = G_A_BYTES + G_B_BYTES;
constexpr int G_THREADS = 192;
constexpr int G_CTAS_PER_SM = 2;
constexpr uint32_t G_TMEM_COLS = 256;
constexpr int G_MAX_FLUSH = 2;  // chunks are at most 2 K-slices (both resident in the ring)
constexpr size_t G_SMEM = (size_t)G_STAGES * G_STAGE_BYTES + 1024 + 256;

struct GroupProblem {  // aligned as its CUtensorMap members
    CUtensorMap mapA[2];  // split Ibar, ping-pong buffers
    CUtensorMap mapW;     // split W^T
    int64_t N;            // cells per group
    int64_t rows;         // groups * N
    int64_t tile_begin;   // first global tile index of this problem
    int m_tiles, n_tiles;
    int Mout, kpad, kblocks, bn, flush, groups;
    uint32_t idesc;
    int fp16;
    int cur;              // buffer holding the current Ibar
    int relax, residual;
    const float* rs;      // [rows_pad] row scales (FP16 mode) or null
    const float* rs_inv;
    const float* cs_inv;  // [mpad] column unscale (FP16 mode) or null
    const float* B;       // [rows] source (null: no update)
    const float* lam;     // [groups] albedo
    float* S32;           // [groups][Mout][N], FP32 (the source iteration)
    double* S64;          // [groups][Mout][N], FP64 (host-buffer calls); used instead of S32 when set
    uint16_t* a[2];       // [rows_pad][2*kpad] interleaved split rows
    unsigned long long* resid;  // residual bits of this problem's step
};

__device__ __forceinline__ int find_problem(const GroupProblem* probs, int nprob, int64_t t)
{
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (probs[mid].tile_begin <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(G_THREADS, G_CTAS_PER_SM)
group_kernel(const GroupProblem* __restrict__ probs, int nprob, int64_t total_tiles, int* flag)
{
    using namespace rts_ptx;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + G_STAGES * G_STAGE_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * G_STAGES + 4);
    const uint32_t smem_base = smem_u32(smem);
    const uint32_t bar_base = smem_u32(bars);
    auto full_bar = [&](int s) { return bar_base + 8u * s; };
    auto empty_bar = [&](int s) { return bar_base + 8u * (G_STAGES + s); };
    auto acc_full_bar = [&](int a) { return bar_base + 8u * (2 * G_STAGES + a); };
    auto acc_empty_bar = [&](int a) { return bar_base + 8u * (2 * G_STAGES + 2 + a); };

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < G_STAGES; ++s) {
            mbar_init(full_bar(s), 1);
            mbar_init(empty_bar(s), 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(acc_full_bar(a), 1);
            mbar_init(acc_empty_bar(a), 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(smem_u32(tmem_slot), G_TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const bool live = *(volatile int*)flag == 0;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0 && live) {
            uint32_t it = 0;
            bool ok = true;
            for (int64_t t = blockIdx.x; t < total_tiles && ok; t += gridDim.x) {
                const GroupProblem& P = probs[find_problem(probs, nprob, t)];
                const int64_t lt = t - P.tile_begin;
                const int n_tiles = P.n_tiles, nkb = P.kblocks, bn = P.bn;
                const int m0 = (int)(lt / n_tiles) * G_BM, n0 = (int)(lt % n_tiles) * bn;
                const void* mapA = &P.mapA[P.cur];
                const void* mapW = &P.mapW;
                const uint32_t tx = (uint32_t)(G_A_BYTES + bn * 128);
                for (int kb = 0; kb < nkb; ++kb, ++it) {
                    const int s = (int)(it % G_STAGES);
                    if (it >= (uint32_t)G_STAGES &&
                        !mbar_wait(empty_bar(s), ((it / G_STAGES) - 1) & 1, flag, FLAG_WAIT_PRODUCER)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(full_bar(s), tx);
                    const uint32_t sa = smem_base + s * G_STAGE_BYTES;
                    tma_load_2d(sa, mapA, kb * 64, m0, full_bar(s));
                    tma_load_2d(sa + G_A_BYTES, mapW, kb * 64, n0, full_bar(s));
                }
            }
            // no copy may still be in flight when the CTA exits
            for (uint32_t i = (it > (uint32_t)G_STAGES ? it - G_STAGES : 0); i < it; ++i)
                mbar_wait(full_bar(i % G_STAGES), (i / G_STAGES) & 1, flag, FLAG_WAIT_PRODUCER);
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0 && live) {
            uint32_t it = 0, ch = 0;  // K-slice and chunk counters (across tiles)
            bool ok = true;
            for (int64_t t = blockIdx.x; t < total_tiles && ok; t += gridDim.x) {
                const GroupProblem& P = probs[find_problem(probs, nprob, t)];
                const uint32_t idesc = P.idesc;
                const int nkb = P.kblocks, flush = P.flush;
                for (int kb0 = 0; kb0 < nkb && ok; kb0 += flush, ++ch) {
                    const int f = min(flush, nkb - kb0);
                    const int a = ch & 1;
                    const uint32_t acc = tmem + 128u * a;
                    if (ch >= 2 && !mbar_wait(acc_empty_bar(a), ((ch >> 1) - 1) & 1, flag, FLAG_WAIT_MMA)) {
                        ok = false;
                        break;
                    }
                    uint32_t ad[G_MAX_FLUSH], bd[G_MAX_FLUSH];
                    for (int j = 0; j < f; ++j) {
                        const uint32_t i2 = it + j;
                        const int s = (int)(i2 % G_STAGES);
                        if (!mbar_wait(full_bar(s), (i2 / G_STAGES) & 1, flag, FLAG_WAIT_MMA)) {
                            ok = false;
                            break;
                        }
                        ad[j] = smem_base + s * G_STAGE_BYTES;
                        bd[j] = ad[j] + G_A_BYTES;
                    }
                    if (!ok) break;
                    tc_fence_after();
                    const uint64_t hi0 = 0, hi1 = 32 >> 4, lo0 = 64 >> 4, lo1 = 96 >> 4;
                    // cross products first (the accumulator starts from zero), hi*hi last
                    for (int j = 0; j < f; ++j) {
                        const uint64_t A = smem_desc_sw128(ad[j]), Bd = smem_desc_sw128(bd[j]);
                        umma_f16(acc, A + hi0, Bd + lo0, idesc, j != 0 ? 1u : 0u);
                        umma_f16(acc, A + lo0, Bd + hi0, idesc, 1u);
                        umma_f16(acc, A + hi1, Bd + lo1, idesc, 1u);
                        umma_f16(acc, A + lo1, Bd + hi1, idesc, 1u);
                    }
                    for (int j = 0; j < f; ++j) {
                        const uint64_t A = smem_desc_sw128(ad[j]), Bd = smem_desc_sw128(bd[j]);
                        umma_f16(acc, A + hi0, Bd + hi0, idesc, 1u);
                        umma_f16(acc, A + hi1, Bd + hi1, idesc, 1u);
                    }
                    for (int j = 0; j < f; ++j) umma_commit(empty_bar((int)((it + j) % G_STAGES)));
                    umma_commit(acc_full_bar(a));
                    it += f;
                }
            }
        }
    } else {
        // ------------------------------------------------------------ epilogue warps
        const int q = warp & 3;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        uint32_t ch = 0;
        bool ok = live;
        for (int64_t t = blockIdx.x; t < total_tiles && ok; t += gridDim.x) {
            const GroupProblem& P = probs[find_problem(probs, nprob, t)];
            // tile parameters, read once into registers
            const int nkb = P.kblocks, flush = P.flush, bn = P.bn, ng = bn >> 4;
            const int nchunks = (nkb + flush - 1) / flush;
            const int64_t lt = t - P.tile_begin;
            const int m_tile = (int)(lt / P.n_tiles), n_tile = (int)(lt % P.n_tiles);
            float run[128];
#pragma unroll
            for (int j = 0; j < 128; ++j) run[j] = 0.0f;
            uint32_t acc = 0;
            for (int c = 0; c < nchunks; ++c, ++ch) {
                const int a = ch & 1;
                acc = tmem + 128u * a + lane_off;
                bool got = true;
                if (lane == 0) got = mbar_wait(acc_full_bar(a), (ch >> 1) & 1, flag, FLAG_WAIT_EPILOGUE);
                if (!__shfl_sync(0xffffffffu, got ? 1 : 0, 0)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                // 32 columns per load-and-wait
#pragma unroll
                for (int g = 0; g < 8; g += 2) {
                    if (g + 1 < ng) {
                        float v[32];
                        tmem_ld32(acc + 16u * g, v);
#pragma unroll
                        for (int j = 0; j < 32; ++j) run[16 * g + j] += v[j];
                    } else if (g < ng) {
                        float v[16];
                        tmem_ld16(acc + 16u * g, v);
#pragma unroll
                        for (int j = 0; j < 16; ++j) run[16 * g + j] += v[j];
                    }
                }
                if (c + 1 < nchunks) {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(acc_empty_bar(a));
                }
            }
            if (!ok) break;
            // the finished sums go back into the last accumulator, which this
            // warp keeps until the epilogue below has read them
#pragma unroll
            for (int g = 0; g < 8; ++g) {
                if (g < ng) {
                    float v[16];
#pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] = run[16 * g + j];
                    tmem_st16(acc + 16u * g, v);
                }
            }
            tmem_wait_st();

            // ---- fused epilogue
            const int64_t r = (int64_t)m_tile * G_BM + q * 32 + lane;
            const int64_t Nc = P.N;
            const int Mout = P.Mout, kpad = P.kpad;
            const bool in_row = r < P.rows;
            const int64_t grp = in_row ? r / Nc : 0;
            const int64_t cc = in_row ? r - grp * Nc : 0;
            const bool fp16 = P.fp16 != 0;
            const bool relax = P.relax != 0, residual = P.residual != 0;
            const float* __restrict__ cs_inv = P.cs_inv;
            const float rinv = (fp16 && in_row) ? P.rs_inv[r] : 1.0f;
            const float rsc = (fp16 && in_row) ? P.rs[r] : 1.0f;
            const bool has_B = P.B != nullptr;
            const float lam = (in_row && has_B) ? P.lam[grp] : 1.0f;
            const float bterm = (in_row && has_B) ? (1.0f - lam) * P.B[r] : 0.0f;
            float* __restrict__ S = P.S32 ? P.S32 + grp * (int64_t)Mout * Nc + cc : nullptr;
            double* __restrict__ S64 = P.S64 ? P.S64 + grp * (int64_t)Mout * Nc + cc : nullptr;
            const int cur = P.cur;
            const uint16_t* __restrict__ arow = P.a[cur] + r * 2 * (int64_t)kpad;
            uint16_t* __restrict__ nrow = P.a[cur ^ 1] + r * 2 * (int64_t)kpad;
            unsigned long long* resid = P.resid;
            const int kbase = n_tile * bn;
            float rmax = 0.0f;
            bool overflow = false;

            // global loads of group g+1 are issued before group g is processed
            float old_n[16];
            uint4 rh_n[2], rl_n[2];
#define RTS_EPI_LOAD(G)                                                                                         \
    do {                                                                                                        \
        const int k0_ = kbase + 16 * (G);                                                                       \
        const bool live_ = in_row && k0_ < Mout;                                                                \
        _Pragma("unroll") for (int j = 0; j < 16; ++j) {                                                        \
            const bool kj = live_ && k0_ + j < Mout;                                                            \
            old_n[j] = (kj && residual && S) ? S[(int64_t)(k0_ + j) * Nc] : 0.0f;                              \
        }                                                                                                       \
        if (live_ && relax && k0_ < kpad) {                                                                     \
            const uint4* src_ = reinterpret_cast<const uint4*>(arow + rts_ptx::ilv_hi(k0_));                    \
            rh_n[0] = src_[0];                                                                                  \
            rh_n[1] = src_[1];                                                                                  \
            rl_n[0] = src_[4];                                                                                  \
            rl_n[1] = src_[5];                                                                                  \
        } else {                                                                                                \
            rh_n[0] = rh_n[1] = rl_n[0] = rl_n[1] = make_uint4(0, 0, 0, 0);                                     \
        }                                                                                                       \
    } while (0)
            RTS_EPI_LOAD(0);
#pragma unroll 1
            for (int g = 0; g < ng; ++g) {
                float old[16];
                uint4 rh[2], rl[2];
#pragma unroll
                for (int j = 0; j < 16; ++j) old[j] = old_n[j];
                rh[0] = rh_n[0];
                rh[1] = rh_n[1];
                rl[0] = rl_n[0];
                rl[1] = rl_n[1];
                if (g + 1 < ng) RTS_EPI_LOAD(g + 1);
                float v[16];
                __syncwarp();
                tmem_ld16(acc + 16u * g, v);
                const int k0 = kbase + 16 * g;
                if (!in_row || k0 >= Mout) continue;
                if (S64) {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (k0 + j < Mout)
                            S64[(int64_t)(k0 + j) * Nc] =
                                (double)(bterm + lam * (v[j] * rinv * (fp16 ? __ldg(cs_inv + k0 + j) : 1.0f)));
                    continue;
                }
                const uint16_t* ph = reinterpret_cast<const uint16_t*>(rh);
                const uint16_t* pl = reinterpret_cast<const uint16_t*>(rl);
                uint16_t nh[16], nl[16];
                const bool do_relax = relax && k0 < kpad;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int k = k0 + j;
                    float xnext = 0.0f;
                    if (k < Mout) {
                        const float cinv = fp16 ? __ldg(cs_inv + k) : 1.0f;
                        const float snew = bterm + lam * (v[j] * rinv * cinv);
                        if (residual) rmax = fmaxf(rmax, fabsf(snew - old[j]));
                        S[(int64_t)k * Nc] = snew;
                        if (do_relax) xnext = 0.5f * join_any(fp16, ph[j], pl[j]) + 0.5f * (snew * rsc);
                    }
                    if (do_relax) {
                        if (fp16 && fabsf(xnext) > 60000.0f) overflow = true;
                        split_any(fp16, xnext, nh[j], nl[j]);
                    }
                }
                if (do_relax) {
                    uint4* dst = reinterpret_cast<uint4*>(nrow + rts_ptx::ilv_hi(k0));
                    dst[0] = make_uint4(pack2(nh[0], nh[1]), pack2(nh[2], nh[3]), pack2(nh[4], nh[5]), pack2(nh[6], nh[7]));
                    dst[1] = make_uint4(pack2(nh[8], nh[9]), pack2(nh[10], nh[11]), pack2(nh[12], nh[13]),
                                        pack2(nh[14], nh[15]));
                    dst[4] = make_uint4(pack2(nl[0], nl[1]), pack2(nl[2], nl[3]), pack2(nl[4], nl[5]), pack2(nl[6], nl[7]));
                    dst[5] = make_uint4(pack2(nl[8], nl[9]), pack2(nl[10], nl[11]), pack2(nl[12], nl[13]),
                                        pack2(nl[14], nl[15]));
                }
            }
#undef RTS_EPI_LOAD
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty_bar((int)((ch - 1) & 1)));
            if (overflow) atomicOr(flag, FLAG_SCALE_OVERFLOW);
            if (residual) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
                if (lane == 0 && rmax > 0.0f)
                    atomicMax(resid, (unsigned long long)__double_as_longlong((double)rmax));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, G_TMEM_COLS);
    }
}

// Flip the ping-pong Ibar buffer of every relaxing problem (launched after
// the step so that a captured graph replays step after step on device).
__global__ void group_flip_kernel(GroupProblem* probs, int nprob)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nprob && probs[p].relax) probs[p].cur ^= 1;
}
