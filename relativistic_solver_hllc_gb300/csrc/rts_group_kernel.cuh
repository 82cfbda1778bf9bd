// rts_group_kernel.cuh -- persistent, grouped tcgen05 contraction of the
// split-precision scattering integral (included by rts_group.cu).
//
// One launch runs one source-iteration step of every problem of a batch: the
// tiles of all problems (128 cells x up to 256 out-directions each; problems
// of different cell and direction counts, phase kernels and precisions) form
// one list that persistent CTAs (one per SM) walk with a fixed stride.
//
// Measured on GB300: one thread issuing M = 128, N = 256 MMAs back to back
// reaches 0.83 of the SM's tensor rate, two threads with an accumulator each
// its full rate.  A CTA runs two issuing warps, each with N up to 256, on
// alternate chunks of the in-direction range of the same tile (split K
// inside the CTA), so that each accumulator is drained while the other
// fills; of the issue schemes measured (one issuer for both accumulators,
// both issuers on every chunk with a column half each) this was the fastest.
//
// Warp roles (19 warps, 608 threads, one CTA per SM):
//   warp 0       TMA producer: A (split Ibar rows) and B (split W rows)
//                K-slices into a 4-stage shared-memory ring;
//   warps 1, 2   MMA issuers (one thread each); warp 1 also owns TMEM
//                (512 columns: one 256-column accumulator per issuer);
//   warps 3..18  drain + epilogue: warp w reads TMEM lanes 32*(w%4).. and a
//                column slice of the tile (a quarter of it, rounded up to
//                16 columns, so narrow tiles keep every warp busy).  After
//                every chunk of `flush` K-slices they add the chunk's
//                accumulator into FP32
//                registers (round-to-nearest adds: the tensor core truncates
//                each accumulate) and release it; the tile's sums go back
//                into its last accumulator, from which the fused epilogue
//                (unscaling, source update, residual, S store, relaxation of
//                Ibar in split form) reads them 8 columns at a time while
//                the other issuer starts the next tile.  Half-way through a
//                tile these warps prefetch the epilogue's inputs into L2.
// Within a chunk the cross products hi*lo and lo*hi (2^-11 or 2^-8 of the
// result) are issued first, while the accumulator is still small, and the two
// hi*hi products last: the truncation then costs about one FP32 ulp of the
// chunk sum per hi*hi MMA.
//
// Relaxed source iterations correct the truncation of the FP32 accumulate
// (each tcgen05.mma rounds toward zero, so the sums come out low by ~1e-7,
// by an amount that depends on how the partial sums grow inside an MMA) with
// a conserved quantity instead of a measured constant: for any W,
//     sum_k (W^T I)_k = sum_j v_j I_j,    v_j = sum_k W[j][k]  (FP64, once).
// E_exact of a step's input needs no pass over it: the relaxation makes the
// next input x' = x/2 + rs S/2, so E_exact' = E_exact/2 + rs (sum_j v_j S_j)/2,
// and the first input's E_exact is computed once at set-up
// (group_energy_init_kernel).  Every relaxed step writes, per cell and per
// epilogue warp, the partial sums of its raw integrals and of v_j S_j into
// per-slot arrays; group_energy_kernel adds the slots, stores each cell's
// delta = E_exact / E_tensor - 1 and advances E_exact, and the next step
// scales that cell's integrals by (1 + delta).  This removes the cell's isotropic bias, the part
// that a relaxed iteration would otherwise compound step after step.  The
// partial sums are exact fixed-point numbers: each block of 8 columns is
// summed in FP32 in column order and rounded to a multiple of a per-row
// power-of-two quantum (2^-43 of a bound on the row's totals), so neither the
// order of the additions nor the tiling of the out-directions changes delta,
// and results stay bit-identical across tile widths and runs.  The kernel is
// compiled with and without this bookkeeping (kEnergy); launches without a
// relaxed problem that uses it run the lighter instantiation.
//
// Every mbarrier wait is bounded (rts_ptx::mbar_wait); a wait that gives up
// sets the device flag, every role stops at its next wait, and the kernel
// drains and exits.

#include <type_traits>

constexpr int G_BM = 128;
constexpr int G_BN = 256;
constexpr int G_STAGES = 4;
constexpr int G_A_BYTES = G_BM * 128;
constexpr int G_B_BYTES = G_BN * 128;
constexpr int G_STAGE_BYTES = G_A_BYTES + G_B_BYTES;
constexpr int G_EPI_WARPS = 16;
constexpr int G_EPI_WARP0 = 3;
constexpr int G_THREADS = (G_EPI_WARP0 + G_EPI_WARPS) * 32;
constexpr int G_CTAS_PER_SM = 1;
constexpr uint32_t G_TMEM_COLS = 512;
constexpr int G_MAX_FLUSH = 2;  // K-slices per chunk
// relaxation row buffers per epilogue warp: G_REL_NB - 1 units are fetched
// ahead of the one being relaxed
constexpr int G_REL_NB = 2;
// ring, accumulator and relaxation barriers (the relaxation's from index 16),
// then the TMEM address
constexpr int G_BAR_BYTES = (8 * (17 + G_REL_NB * G_EPI_WARPS) + 127) / 128 * 128;
constexpr int G_REL_BUF = G_REL_NB * 1024;  // per epilogue warp: buffers of 32 rows x 16 B hi, then 32 rows x 16 B lo
constexpr size_t G_REL_OFF = (size_t)G_STAGES * G_STAGE_BYTES + G_BAR_BYTES;
constexpr size_t G_SMEM = G_REL_OFF + (size_t)G_EPI_WARPS * G_REL_BUF + 1024;
static_assert(G_SMEM <= 227 * 1024, "shared memory per CTA");

struct GroupProblem {  // aligned as its CUtensorMap members
    CUtensorMap mapA[2];  // split Ibar, ping-pong buffers
    CUtensorMap mapW;     // split W^T
    CUtensorMap mapR[2];  // split Ibar in relaxation boxes (8 columns x 32 rows), ping-pong buffers
    int64_t N;            // cells per group
    int64_t ldS;          // row pitch of S32 / S64 in cells (>= N; N unless the output is a cell range of a wider S)
    int64_t rows;         // groups * N
    int64_t tile_begin;   // first global tile index of this problem in the launch
    int64_t tile_off;     // the problem's own first tile in this launch (a step may span launches)
    int m_tiles, n_tiles;
    int Mout, kpad, kblocks, bn, flush, groups;
    int order;            // tile order: 0 the column tiles of a row tile in turn, 1 the row tiles of a column tile
    uint32_t idesc;
    float bias;           // relative correction of the truncation bias of the sums
    int fp16;
    int tf32;             // split TF32 operands (kind::tf32, 16 in-directions per K-slice)
    int sw;               // columns per epilogue column slice: a quarter of bn rounded up to 16 (at most 64)
    int cur;              // buffer holding the current Ibar
    int relax, residual;
    int flip;             // the step ends in this launch: flip the ping-pong Ibar buffer after it
    const float* rs;      // [rows_pad] row scales (FP16 mode) or null
    const float* rs_inv;
    const float* cs_inv;  // [mpad] column unscale (FP16 mode) or null
    const float* B;       // [rows] source (null: no update)
    const float* lam;     // [groups] albedo
    float* S32;           // [groups][Mout][N], FP32 (the source iteration)
    double* S64;          // [groups][Mout][N], FP64 (host-buffer calls); used instead of S32 when set
    uint16_t* a[2];       // [rows_pad][2*kpad] interleaved split rows
    unsigned long long* resid;  // residual bits of this problem's step
    // energy-conservation correction of relaxed steps (null: none)
    const float* vrow;    // [kpad + 4] v_j = sum_k W[j][k], 0 past M; vrow[kpad] = q0 (below), then c, D, 1/c:
                          // c the mean of the v_j, D = sum_j (v_j - c); output column Mout holds
                          // sum_j (v_j - c) raw_j
    int4* part;           // [n_tiles * 4][rows_pad] per-slot partials in quanta (high, low parts):
                          // sum_j v_j rs S_j, then sum_k raw_k
    double* ex;           // [rows_pad] sum_j v_j x_j of the current input, in quanta
    float* delta;         // [rows_pad] per-cell correction of the next step (0: none yet)
    const float* rsb;     // [rows_pad] power of two with rsb * 2 max(|Ibar|, |B|) < 2^14 (all modes)
};

// Scale of a row's partial sums: q0 * (the row's scale for the unscaled
// formats), a power of two with (scale * bound of the row's totals) <= 2^21.
// q0 = 2^(7 - ceil(log2 sum_jk |W_jk|)) comes with vrow; values in the units
// the epilogue sees are below 2^14 (FP16, scaled) or 2^14 / rsb (BF16,
// TF32).  0 when out of FP32 range (no correction for the row).
__device__ __forceinline__ float energy_scale(const GroupProblem& P, int64_t r, bool fp16)
{
    const float q = P.vrow[P.kpad] * (fp16 ? 1.0f : P.rsb[r]);
    return (q > 0.0f && q < 3.0e38f) ? q : 0.0f;
}

// Adds y (|y| <= 2^21) to an exact fixed-point sum kept as integer high and
// low parts, hi + lo * 2^-22 (units of 1 and 2^-22): adding 1.5 * 2^23 rounds
// to an integer in FP32, and the remainder, scaled by 2^22 (exact), is
// rounded the same way.  No conversion instructions; the sum of such parts is
// exact in any order.
__device__ __forceinline__ void fixed_add(float y, int& hi, int& lo)
{
    constexpr float MAGIC = 12582912.0f;  // 1.5 * 2^23
    const float t = y + MAGIC;
    const float r = y - (t - MAGIC);
    const float t2 = fmaf(r, 4194304.0f, MAGIC);
    hi += __float_as_int(t) - __float_as_int(MAGIC);
    lo += __float_as_int(t2) - __float_as_int(MAGIC);
}

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

// Row and column tile of a problem's tile lt (0 <= lt < m_tiles * n_tiles).
__device__ __forceinline__ void tile_coords(const GroupProblem& P, int64_t lt, int& m_tile, int& n_tile)
{
    if (P.order) {
        m_tile = (int)(lt % P.m_tiles);
        n_tile = (int)(lt / P.m_tiles);
    } else {
        m_tile = (int)(lt / P.n_tiles);
        n_tile = (int)(lt % P.n_tiles);
    }
}

// Relaxation of 8 columns of one split row in place (shared memory):
// Ibar' = 0.5 Ibar + 0.5 * (rs * S), split again into hi + lo; columns at or
// past `nk` become zero (the padding of the split rows).  Returns true when
// an FP16 value leaves the range the row scale allows.
template <bool kFp16>
__device__ __forceinline__ bool relax8(uint4* hp, uint4* lp, const float (&snew)[8], float hrsc, int nk)
{
    const uint4 rh = *hp, rl = *lp;
    const uint32_t hw[4] = {rh.x, rh.y, rh.z, rh.w};
    const uint32_t lw[4] = {rl.x, rl.y, rl.z, rl.w};
    uint32_t nh[4], nl[4];
    float amax = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
        const float2 i2 = rts_ptx::join2_any(kFp16, hw[j >> 1], lw[j >> 1]);
        const float x0 = (j < nk) ? fmaf(snew[j], hrsc, 0.5f * i2.x) : 0.0f;
        const float x1 = (j + 1 < nk) ? fmaf(snew[j + 1], hrsc, 0.5f * i2.y) : 0.0f;
        if (kFp16) amax = fmaxf(amax, fmaxf(fabsf(x0), fabsf(x1)));
        rts_ptx::split2_any(kFp16, x0, x1, nh[j >> 1], nl[j >> 1]);
    }
    *hp = make_uint4(nh[0], nh[1], nh[2], nh[3]);
    *lp = make_uint4(nl[0], nl[1], nl[2], nl[3]);
    return amax > 60000.0f;
}

// The same for 4 columns of a split TF32 row (hi and lo as FP32, no scale).
__device__ __forceinline__ void relax4_tf32(float4* hp, float4* lp, const float* snew, float hrsc, int nk)
{
    const float4 h = *hp, l = *lp;
    const float hv[4] = {h.x, h.y, h.z, h.w}, lv[4] = {l.x, l.y, l.z, l.w};
    float nh[4], nl[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float x = (j < nk) ? fmaf(snew[j], hrsc, 0.5f * (hv[j] + lv[j])) : 0.0f;
        rts_ptx::split_tf32(x, nh[j], nl[j]);
    }
    *hp = make_float4(nh[0], nh[1], nh[2], nh[3]);
    *lp = make_float4(nl[0], nl[1], nl[2], nl[3]);
}

template <bool kEnergy>
__global__ void __launch_bounds__(G_THREADS, 1)
group_kernel(const GroupProblem* __restrict__ probs, int nprob, int64_t total_tiles, int* flag)
{
    using namespace rts_ptx;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + G_STAGES * G_STAGE_BYTES);  // G_BAR_BYTES
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 16 + G_REL_NB * G_EPI_WARPS);
    const uint32_t smem_base = smem_u32(smem);
    const uint32_t bar_base = smem_u32(bars);
    auto full_bar = [&](int s) { return bar_base + 8u * s; };
    auto empty_bar = [&](int s) { return bar_base + 8u * (G_STAGES + s); };
    auto acc_full_bar = [&](int a) { return bar_base + 8u * (2 * G_STAGES + a); };
    auto acc_empty_bar = [&](int a) { return bar_base + 8u * (2 * G_STAGES + 2 + a); };
    // relaxation row buffers: barrier of buffer b of epilogue warp w
    auto rel_bar = [&](int w, uint32_t b) { return bar_base + 8u * (16 + G_REL_NB * w + (int)b); };

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < G_STAGES; ++s) {
            mbar_init(full_bar(s), 1);
            mbar_init(empty_bar(s), 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(acc_full_bar(a), 1);
            mbar_init(acc_empty_bar(a), G_EPI_WARPS);
        }
        for (int w = 0; w < G_EPI_WARPS; ++w)
            for (int b = 0; b < G_REL_NB; ++b) mbar_init(rel_bar(w, (uint32_t)b), 1);
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
                const int64_t lt = t - P.tile_begin + P.tile_off;
                const int nkb = P.kblocks, bn = P.bn;
                int m_tile, n_tile;
                tile_coords(P, lt, m_tile, n_tile);
                const int m0 = m_tile * G_BM, n0 = n_tile * bn;
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
    } else if (warp == 1 || warp == 2) {
        // ------------------------------------------------------------ MMA issuers
        const uint32_t me = (uint32_t)(warp - 1);
        if (lane == 0 && live) {
            const uint32_t acc = tmem + 256u * me;
            uint32_t gsl = 0, gch = 0;  // K-slice and chunk counters of this CTA (across tiles)
            bool ok = true;
            for (int64_t t = blockIdx.x; t < total_tiles && ok; t += gridDim.x) {
                const GroupProblem& P = probs[find_problem(probs, nprob, t)];
                const uint32_t idesc = P.idesc;
                const int nkb = P.kblocks, flush = P.flush;
                const int nchunks = (nkb + flush - 1) / flush;
                // the chunk loop, compiled once per MMA kind
                auto chunks = [&](auto tf32c) {
                    constexpr bool tf32 = decltype(tf32c)::value;
                    auto mma = [&](uint64_t a, uint64_t b, uint32_t accumulate) {
                        if (tf32)
                            umma_tf32(acc, a, b, idesc, accumulate);
                        else
                            umma_f16(acc, a, b, idesc, accumulate);
                    };
                    for (int c = 0; c < nchunks; ++c) {
                        const uint32_t g = gch + (uint32_t)c;
                        if ((g & 1u) != me) continue;
                        const int kb0 = c * flush;
                        const int f = min(flush, nkb - kb0);
                        if (g >= 2 && !mbar_wait(acc_empty_bar(me), ((g >> 1) - 1) & 1, flag, FLAG_WAIT_MMA)) {
                            ok = false;
                            break;
                        }
                        uint32_t ad[G_MAX_FLUSH], st[G_MAX_FLUSH];
                        for (int j = 0; j < f; ++j) {
                            const uint32_t i2 = gsl + (uint32_t)(kb0 + j);
                            st[j] = i2 % G_STAGES;
                            if (!mbar_wait(full_bar((int)st[j]), (i2 / G_STAGES) & 1, flag, FLAG_WAIT_MMA)) {
                                ok = false;
                                break;
                            }
                            ad[j] = smem_base + st[j] * G_STAGE_BYTES;
                        }
                        if (!ok) break;
                        tc_fence_after();
                        const uint64_t hi0 = 0, hi1 = 32 >> 4, lo0 = 64 >> 4, lo1 = 96 >> 4;
                        // cross products first (the accumulator starts from zero), hi*hi last
                        for (int j = 0; j < f; ++j) {
                            const uint64_t A = smem_desc_sw128(ad[j]), Bd = smem_desc_sw128(ad[j] + G_A_BYTES);
                            mma(A + hi0, Bd + lo0, j != 0 ? 1u : 0u);
                            mma(A + lo0, Bd + hi0, 1u);
                            mma(A + hi1, Bd + lo1, 1u);
                            mma(A + lo1, Bd + hi1, 1u);
                        }
                        for (int j = 0; j < f; ++j) {
                            const uint64_t A = smem_desc_sw128(ad[j]), Bd = smem_desc_sw128(ad[j] + G_A_BYTES);
                            mma(A + hi0, Bd + hi0, 1u);
                            mma(A + hi1, Bd + hi1, 1u);
                        }
                        for (int j = 0; j < f; ++j) umma_commit(empty_bar((int)st[j]));
                        umma_commit(acc_full_bar((int)me));
                    }
                };
                if (P.tf32)
                    chunks(std::true_type{});
                else
                    chunks(std::false_type{});
                gch += (uint32_t)nchunks;
                gsl += (uint32_t)nkb;
            }
        }
    } else {
        // ------------------------------------------------------------ drain + epilogue warps
        const int q = warp & 3;                    // TMEM lane quarter
        const int cs = (warp - G_EPI_WARP0) >> 2;  // column slice of the tile
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        const int ew = warp - G_EPI_WARP0;
        uint8_t* rbuf = smem + G_REL_OFF + (size_t)ew * G_REL_BUF;
        const uint32_t rbuf_s = smem_u32(rbuf);
        uint32_t rel_issued = 0, rel_used = 0;  // relaxation row blocks fetched / consumed by this warp
        uint32_t gch = 0;
        bool ok = live;
        for (int64_t t = blockIdx.x; t < total_tiles && ok; t += gridDim.x) {
            const GroupProblem& P = probs[find_problem(probs, nprob, t)];
            const int nkb = P.kblocks, flush = P.flush, bn = P.bn;
            const int nchunks = (nkb + flush - 1) / flush;
            const int sw = P.sw;                         // columns per slice (multiple of 16, <= 64)
            const int ncols = min(sw, bn - sw * cs);  // columns of this warp (multiple of 16; <= 0: none)
            const int64_t lt = t - P.tile_begin + P.tile_off;
            int m_tile, n_tile;
            tile_coords(P, lt, m_tile, n_tile);
            float run[64];
#pragma unroll
            for (int j = 0; j < 64; ++j) run[j] = 0.0f;
            uint32_t last_acc = 0;
            int last_a = 0;
            for (int c = 0; c < nchunks; ++c) {
                const uint32_t g = gch + (uint32_t)c;
                const int a = (int)(g & 1u);
                const uint32_t acc = tmem + 256u * (uint32_t)a + lane_off + (uint32_t)(sw * cs);
                bool got = true;
                if (lane == 0) got = mbar_wait(acc_full_bar(a), (g >> 1) & 1, flag, FLAG_WAIT_EPILOGUE);
                if (!__shfl_sync(0xffffffffu, got ? 1 : 0, 0)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
#pragma unroll
                for (int gi = 0; gi < 4; ++gi) {
                    if (16 * gi < ncols) {
                        float v[16];
                        tmem_ld16(acc + 16u * gi, v);
#pragma unroll
                        for (int j = 0; j < 16; ++j) run[16 * gi + j] += v[j];
                    }
                }
                if (c + 1 < nchunks) {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(acc_empty_bar(a));
                    // a few chunks before the end of the tile, pull the epilogue's
                    // inputs (the previous S and the Ibar rows it relaxes) into L2
                    if (c == max(0, nchunks - 4) && ncols > 0) {
                        const int64_t r = (int64_t)m_tile * G_BM + q * 32 + lane;
                        if (r < P.rows) {
                            const int64_t Nc = P.N, ld = P.ldS;
                            const int Mout = P.Mout, kb0 = n_tile * bn + sw * cs;
                            const int64_t grp = r / Nc;
                            if (P.S32 && P.residual) {
                                const float* Sp = P.S32 + grp * (int64_t)Mout * ld + (r - grp * Nc);
                                for (int j = 0; j < ncols && kb0 + j < Mout; ++j)
                                    prefetch_l2(Sp + (int64_t)(kb0 + j) * ld);
                            }
                            if (P.relax && P.S32 && !P.S64 && kb0 < P.kpad) {
                                const uint16_t* ar = P.a[P.cur] + r * 2 * (int64_t)P.kpad;
                                const int b0 = kb0 >> 5, b1 = min(kb0 + ncols - 1, P.kpad - 1) >> 5;
                                for (int b = b0; b <= b1; ++b) prefetch_l2(ar + 64 * (int64_t)b);
                            }
                        }
                    }
                } else {
                    // the finished sums go back into the last accumulator, which
                    // this warp keeps until the epilogue below has read them
#pragma unroll
                    for (int gi = 0; gi < 4; ++gi) {
                        if (16 * gi < ncols) {
                            float v[16];
#pragma unroll
                            for (int j = 0; j < 16; ++j) v[j] = run[16 * gi + j];
                            tmem_st16(acc + 16u * gi, v);
                        }
                    }
                    tmem_wait_st();
                    last_acc = acc;
                    last_a = a;
                }
            }
            gch += (uint32_t)nchunks;
            if (!ok) break;
            auto release_last = [&]() {
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(acc_empty_bar(last_a));
            };
            if (ncols <= 0) {
                release_last();
                continue;
            }

            // ---- fused epilogue, reading the sums back 8 columns at a time:
            //   S = (1 - lam) B + lam * rs_inv[row] * cs_inv[k] * acc
            //   Ibar' = 0.5 Ibar + 0.5 rs[row] * S   (relaxation, split again)
            const int64_t r = (int64_t)m_tile * G_BM + q * 32 + lane;
            const int64_t Nc = P.N, ld = P.ldS;
            const int Mout = P.Mout;
            const bool in_row = r < P.rows;
            const int64_t grp = in_row ? r / Nc : 0;
            const int64_t cc = in_row ? r - grp * Nc : 0;
            const bool fp16 = P.fp16 != 0;
            // the energy instantiation runs relaxed source-iteration steps only
            const bool relax = kEnergy || P.relax != 0, residual = kEnergy || P.residual != 0;
            const float* __restrict__ cs_inv = P.cs_inv;
            const bool has_B = kEnergy || P.B != nullptr;
            const float lam = (in_row && has_B) ? P.lam[grp] : 1.0f;
            const float lr = lam * ((fp16 && in_row) ? P.rs_inv[r] : 1.0f);
            const float bterm = (in_row && has_B) ? (1.0f - lam) * P.B[r] : 0.0f;
            const float hrsc = 0.5f * ((fp16 && in_row) ? P.rs[r] : 1.0f);
            const bool want_rel = kEnergy || (relax && P.S64 == nullptr);  // relax implies Mout == M <= kpad
            // energy-conservation correction (relaxed steps): this cell's delta
            // from the previous step; the partial sums of this one.
            const bool ewarp = kEnergy && want_rel && P.part != nullptr;
            const float qrow = (ewarp && in_row) ? energy_scale(P, r, fp16) : 0.0f;
            const bool cons = qrow > 0.0f;
            const float bias = P.bias + (cons ? P.delta[r] : 0.0f);
            // the partial sums: sum_k raw_k in fixed point, and the raw value
            // of the extra column Mout (sum_j (v_j - c) raw_j) where this warp
            // holds it; group_energy_kernel derives sum_j v_j S_j from them
            int th = 0, tl = 0;
            float raw_e = 0.0f;
            const int kbase = n_tile * bn + sw * cs;
            float* __restrict__ S = P.S32 ? P.S32 + grp * (int64_t)Mout * ld + cc : nullptr;
            // (the energy instantiation runs relaxed source iterations, whose output is S32)
            double* __restrict__ S64 = (!kEnergy && P.S64) ? P.S64 + grp * (int64_t)Mout * ld + cc : nullptr;
            // The relaxation's split rows move by TMA in units of 16 B hi and
            // 16 B lo of each of the warp's 32 rows (8 columns of a 16-bit
            // split, 4 of a TF32 split): a 2-D box load into one of two
            // shared-memory buffers per warp, one unit ahead, and after the
            // update a box store back into the other ping-pong buffer.  A buffer
            // is refilled only once the store that read it has finished reading
            // (rows 4*kpad bytes apart would otherwise cost a line per lane on
            // every access).
            float rmax = 0.0f;
            bool overflow = false;
            // the steps, compiled once per split format (columns per relaxation unit)
            auto run_steps = [&](auto tf32c) {
                constexpr bool tf32 = decltype(tf32c)::value;
                constexpr int ucols = tf32 ? 4 : 8;
                const int row0 = m_tile * G_BM + q * 32;
                const void* map_in = &P.mapR[P.cur];
                const void* map_out = &P.mapR[P.cur ^ 1];
                // units of this warp's columns that hold outputs
                const int u_real = want_rel ? max(0, min(ncols, Mout - kbase) + ucols - 1) / ucols : 0;
                auto unit_x = [&](int u) {  // box column (16-bit units) of unit u's high parts
                    const int k0 = kbase + u * ucols;
                    return tf32 ? (k0 >> 4) * 64 + (k0 & 15) * 2 : (k0 >> 5) * 64 + (k0 & 31);
                };
                int u_next = 0;  // next unit to fetch
                auto pump = [&](int u_cons) {  // keep G_REL_NB - 1 units fetched beyond the one being consumed
                    while (u_next < u_real && u_next <= u_cons + (G_REL_NB - 1)) {
                        if (lane == 0) {
                            const uint32_t b = rel_issued % G_REL_NB, dst = rbuf_s + b * 1024u;
                            const int x = unit_x(u_next);
                            bulk_wait_read0();  // the store that last read this buffer
                            mbar_expect_tx(rel_bar(ew, b), 1024);
                            tma_load_2d(dst, map_in, x, row0, rel_bar(ew, b));
                            tma_load_2d(dst + 512u, map_in, x + 32, row0, rel_bar(ew, b));
                        }
                        ++rel_issued;
                        ++u_next;
                    }
                };
                // previous S of a block of 8 columns, loaded one block ahead
                auto load_old = [&](int e0, float (&o)[8]) {
                    const int k0 = kbase + e0;
                    const int nk = min(8, Mout - k0);
                    if (in_row && nk > 0 && residual && S && e0 < ncols) {
                        const float* sp = S + (int64_t)k0 * ld;
    #pragma unroll
                        for (int j = 0; j < 8; ++j, sp += ld) o[j] = j < nk ? *sp : 0.0f;
                    } else {
    #pragma unroll
                        for (int j = 0; j < 8; ++j) o[j] = 0.0f;
                    }
                };
                float old_next[8];
                load_old(0, old_next);
                pump(-1);
    #pragma unroll 1
                for (int e0 = 0; e0 < ncols; e0 += 8) {
                    const int k0 = kbase + e0;
                    const int nk = min(8, Mout - k0);  // valid columns of this block (same for all lanes)
                    const bool live_k = in_row && nk > 0;
                    float old[8];
    #pragma unroll
                    for (int j = 0; j < 8; ++j) old[j] = old_next[j];
                    load_old(e0 + 8, old_next);
                    float cin[8];
                    if (fp16) {
                        const float4 c0 = __ldg(reinterpret_cast<const float4*>(cs_inv + k0));
                        const float4 c1 = __ldg(reinterpret_cast<const float4*>(cs_inv + k0) + 1);
                        cin[0] = c0.x, cin[1] = c0.y, cin[2] = c0.z, cin[3] = c0.w;
                        cin[4] = c1.x, cin[5] = c1.y, cin[6] = c1.z, cin[7] = c1.w;
                    } else {
    #pragma unroll
                        for (int j = 0; j < 8; ++j) cin[j] = 1.0f;
                    }
                    float v[8];
                    tmem_ld8(last_acc + (uint32_t)e0, v);
                    float snew[8];
                    float eb = 0.0f;  // these columns' raw integrals, in column order
    #pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const float raw = v[j] * cin[j];  // cin is a power of two: exact
                        snew[j] = fmaf(fmaf(raw, bias, raw), lr, bterm);
                        if (kEnergy && j < nk) eb += raw;
                        if (kEnergy && j == nk) raw_e = raw;  // column Mout (one block of one warp)
                    }
                    // blocks of 8 columns start at multiples of 8 of the out-directions
                    if (kEnergy && cons && live_k) fixed_add(eb * qrow, th, tl);
                    if (live_k) {
                        if (S64) {
                            double* dp = S64 + (int64_t)k0 * ld;
    #pragma unroll
                            for (int j = 0; j < 8; ++j, dp += ld)
                                if (j < nk) *dp = (double)snew[j];
                        } else {
                            float* sp = S + (int64_t)k0 * ld;
    #pragma unroll
                            for (int j = 0; j < 8; ++j, sp += ld)
                                if (j < nk) {
                                    *sp = snew[j];
                                    rmax = fmaxf(rmax, fabsf(snew[j] - old[j]));
                                }
                        }
                    }
                    // fetch one unit ahead only now: the buffer it fills was read by
                    // the previous step's store, which has had the TMEM read and the
                    // S stores above to finish, so lane 0 rarely waits on it
                    pump(e0 / ucols);
                    // this step's units: wait for the load, relax this lane's row in
                    // place (rows outside the problem stay unchanged), store the box
                    // into the other ping-pong buffer
                    bool stop = false;
                    for (int ui = 0; ui < 8 / ucols; ++ui) {
                        const int u = e0 / ucols + ui;
                        if (u >= u_real) break;
                        const uint32_t b = rel_used % G_REL_NB;
                        const bool got =
                            mbar_wait(rel_bar(ew, b), (rel_used / G_REL_NB) & 1u, flag, FLAG_WAIT_EPILOGUE);
                        ++rel_used;
                        if (!__all_sync(0xffffffffu, got)) {
                            stop = true;
                            break;
                        }
                        uint8_t* rb = rbuf + b * 1024u;
                        const int nku = min(ucols, Mout - (kbase + u * ucols));
                        if (in_row) {
                            if (tf32) {
                                relax4_tf32(reinterpret_cast<float4*>(rb + 16 * lane),
                                            reinterpret_cast<float4*>(rb + 512 + 16 * lane), snew + 4 * ui, hrsc, nku);
                            } else {
                                uint4* hp = reinterpret_cast<uint4*>(rb + 16 * lane);
                                uint4* lp = reinterpret_cast<uint4*>(rb + 512 + 16 * lane);
                                if (fp16)
                                    overflow |= relax8<true>(hp, lp, snew, hrsc, nku);
                                else
                                    relax8<false>(hp, lp, snew, hrsc, nku);
                            }
                        }
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0) {
                            const int x = unit_x(u);
                            tma_store_2d(map_out, x, row0, rbuf_s + b * 1024u);
                            tma_store_2d(map_out, x + 32, row0, rbuf_s + b * 1024u + 512u);
                            bulk_commit();
                        }
                        pump(u);
                    }
                    if (stop) {
                        ok = false;
                        break;
                    }
                }
            };
            if (P.tf32)
                run_steps(std::true_type{});
            else
                run_steps(std::false_type{});
            release_last();
            if (kEnergy && ewarp && in_row && ok) {  // this slot's partial sums (zero: no correction)
                const int64_t slot = (int64_t)n_tile * 4 + cs;
                P.part[slot * (P.m_tiles * (int64_t)G_BM) + r] = make_int4(cons ? __float_as_int(raw_e) : 0, 0, th, tl);
            }
            if (overflow) atomicOr(flag, FLAG_SCALE_OVERFLOW);
            if (residual) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
                if (lane == 0 && rmax > 0.0f)
                    atomicMax(P.resid, (unsigned long long)__double_as_longlong((double)rmax));
            }
        }
        if (lane == 0) bulk_wait0();  // the relaxation's stores are complete before the CTA exits
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, G_TMEM_COLS);
    }
}

// After a relaxed step: each cell's correction for the next step, from the
// per-slot partial sums of the step (added in a fixed slot order):
// delta = sum_j v_j I_j / sum_k raw_k - 1, or 0 when either sum is not
// positive or the ratio is far from 1 (a W with cancelling signs).
// blockIdx.y: problem; only problems whose step ended in this launch.
__global__ void group_energy_kernel(const GroupProblem* __restrict__ probs, int nprob)
{
    const GroupProblem& P = probs[blockIdx.y];
    if (!(P.relax && P.flip && P.part && P.S64 == nullptr)) return;
    const int64_t ld = P.m_tiles * (int64_t)G_BM;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < P.rows;
         r += (int64_t)gridDim.x * blockDim.x) {
        long long et = 0;  // exact: in units of 2^-22 of the row's quantum
        float raw_e = 0.0f;  // held by one slot, zero in the others
        for (int nt = 0; nt < P.n_tiles; ++nt)
            for (int cs = 0; cs < 4; ++cs) {
                if (P.sw * cs >= P.bn) continue;  // a column slice without columns
                const int4 v = P.part[((int64_t)nt * 4 + cs) * ld + r];
                raw_e += __int_as_float(v.x);
                et += ((long long)v.z << 22) + v.w;
            }
        const double q22 = 1.0 / 4194304.0;  // the slots' units, in quanta
        const double ex = P.ex[r];           // sum_j v_j x_j of this step's input, in quanta
        const bool fp16 = P.fp16 != 0;
        const float qrow = energy_scale(P, r, fp16);
        // the step's S_j = (1 + b) lr raw_j + bterm (lr = lam / rs, rs = 1
        // for the unscaled formats), so with v_j = c + d_j
        //   rs sum_j v_j S_j = (1 + b) lam (c sum_j raw_j + sum_j d_j raw_j) + rs bterm sum_j v_j,
        // the raw sums in the units the epilogue sees (scaled by rs)
        const float d_old = P.delta[r];
        const double b1 = 1.0 + (double)(P.bias + (qrow > 0.0f ? d_old : 0.0f));
        const int64_t grp = r / P.N;
        const double lam = (double)P.lam[grp];
        const double bterm = P.B ? (1.0 - lam) * (double)P.B[r] : 0.0;
        const double rs = fp16 ? (double)P.rs[r] : 1.0;
        const double c = (double)P.vrow[P.kpad + 1], V = c * P.Mout + (double)P.vrow[P.kpad + 2];
        const double ev = b1 * lam * (c * ((double)et * q22) + (double)raw_e * qrow) + rs * bterm * V * qrow;
        float d = 0.0f;
        if (ex > 0.0 && et > 0) {
            const double g = ex / ((double)et * q22) - 1.0;
            if (fabs(g) < 1e-4) d = (float)g;
        }
        P.delta[r] = d;
        // the next input is x / 2 + rs S / 2
        P.ex[r] = qrow > 0.0f ? 0.5 * ex + 0.5 * ev : 0.0;
    }
}

// sum_j v_j x_j of every row of the current split input, in the quanta of
// energy_scale (FP64, once per set-up of an iteration): the split values
// joined as the tensor core multiplies them (hi + lo).  A warp per row, its
// lanes on consecutive columns (coalesced), FP64 lane sums reduced in a fixed
// shuffle order.
__global__ void group_energy_init_kernel(const uint16_t* __restrict__ A, int64_t rows, int kpad, int M, int mode,
                                         const float* __restrict__ vrow, const float* __restrict__ rs, double* ex)
{
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= rows) return;  // r is uniform over the warp
    float q = vrow[kpad] * (mode == 1 ? 1.0f : rs[r]);
    if (!(q > 0.0f && q < 3.0e38f)) q = 0.0f;
    double s = 0.0;
    if (mode == 2) {
        const float* row = reinterpret_cast<const float*>(A + r * 4 * (int64_t)kpad);
        for (int j = lane; j < M; j += 32) {
            const int h = (j >> 4) * 32 + (j & 15);
            s += (double)vrow[j] * (double)(row[h] + row[h + 16]);
        }
    } else {
        const uint16_t* row = A + r * 2 * (int64_t)kpad;
        for (int j = lane; j < M; j += 32) {
            const int64_t h = rts_ptx::ilv_hi(j);
            s += (double)vrow[j] * (double)rts_ptx::join_any(mode == 1, row[h], row[h + 32]);
        }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) ex[r] = s * (double)q;
}

// Flip the ping-pong Ibar buffer of every problem whose relaxed step ended in
// this launch (launched after it, so that a captured graph replays step after
// step on the device).
__global__ void group_flip_kernel(GroupProblem* probs, int nprob)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nprob && probs[p].flip) probs[p].cur ^= 1;
}
