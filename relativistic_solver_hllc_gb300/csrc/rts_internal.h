// rts_internal.h -- context state and helpers shared by the library's
// translation units.  Not installed; the public surface is include/rts_scatter.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "rts_scatter.h"

// Error reporting: every entry point returns an rts_status and stores a
// message in the context.  No path calls exit() (the reference's
// CUDA_CALL_FUNC exits the process, cuda/cuda_def.cuh:18-20,31-40).
struct rts_ctx;
int rts_fail(rts_ctx* ctx, int status, const char* fmt, ...);

#define RTS_CUDA_TRY(ctx, call)                                                            \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return rts_fail((ctx), RTS_ERR_CUDA, "%s failed: %s (%s:%d)", #call,           \
                            cudaGetErrorString(e_), __FILE__, __LINE__);                   \
    } while (0)

#define RTS_CHECK_LAUNCH(ctx, what)                                                        \
    do {                                                                                   \
        cudaError_t e_ = cudaGetLastError();                                               \
        if (e_ != cudaSuccess)                                                             \
            return rts_fail((ctx), RTS_ERR_CUDA, "launch of %s failed: %s", (what),        \
                            cudaGetErrorString(e_));                                       \
    } while (0)

#define RTS_REQUIRE(ctx, cond, status, ...)                                                \
    do {                                                                                   \
        if (!(cond)) return rts_fail((ctx), (status), __VA_ARGS__);                        \
    } while (0)

constexpr int64_t RTS_RESID_CAP = 4096;

// Split-precision operands of one source iteration (tensor-core path).
struct rts_batch;
constexpr int RTS_HOST_CHUNKS = 16;  // cell ranges of a pipelined host-buffer call

struct rts_tune_entry {  // autotuned schedule of the tensor-core kernel
    int64_t M = 0;
    int precision = 0, flush = 1;
    int bucket = -1;  // cell-count bucket (rts_cells_bucket); -1: any (tables without buckets)
    int bn = 0, order = 0;
    double ms = 0.0;
};

struct rts_split_state {
    int precision = -1;             // precision of the resident source iteration
    rts_batch* iter = nullptr;      // one-problem batch of the source iteration
    int64_t iter_id = 0;
    // host-buffer calls: one one-problem batch per cell range, pipelined
    // (copy in on `copy_in`, split + contraction on the scattering stream,
    // copy out on `copy_out`)
    rts_batch* chunk[RTS_HOST_CHUNKS] = {};
    int64_t chunk_id[RTS_HOST_CHUNKS] = {};
    int64_t chunk_w_version[RTS_HOST_CHUNKS] = {};
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t ev_start = nullptr, ev_in[RTS_HOST_CHUNKS] = {}, ev_done[RTS_HOST_CHUNKS] = {};
    // reference-compatible asynchronous calls (rts_scattering_async) at a
    // tensor precision: one one-problem batch per stream slot (its split W
    // rows of the slot's out-directions, its outputs), so that calls queued on
    // different streams at the same time (the reference's pair on scattering
    // streams 1 and 2) never share a buffer they write
    rts_batch* slot[RTS_STREAM_COUNT] = {};
    int64_t slot_id[RTS_STREAM_COUNT] = {};
    int64_t slot_start[RTS_STREAM_COUNT] = {};
    int64_t slot_w_version[RTS_STREAM_COUNT] = {};
    int64_t slot_gen[RTS_STREAM_COUNT] = {};   // call_gen the slot's problem was built on
    // ... and their split Ibar rows, which depend on the Illum only: one copy
    // shared by the slots, prepared by a call and reused by the next call on
    // each other slot while the inputs are unchanged (the pair)
    uint16_t* call_a = nullptr;               // [rows_pad][units]
    float* call_rs = nullptr;                 // [2*rows_pad] row scales, inverse
    double* call_sums = nullptr;              // [M][N] FP64 face sums (staging)
    unsigned long long* call_max = nullptr;   // [N] max |face mean| per cell (FP64 bits)
    size_t call_a_bytes = 0, call_rs_bytes = 0, call_sums_bytes = 0, call_max_bytes = 0;
    int call_mode = -1;
    int64_t call_N = 0, call_M = 0;
    int64_t call_gen = 0;                     // bumped when the shared buffers are reallocated
    int64_t call_version = -1;                // inputs_version the rows were prepared from
    int prep_slot = -1;                       // slot whose call prepared them
    bool prep_served[RTS_STREAM_COUNT] = {};  // other slots that have reused them
    cudaEvent_t ev_prep = nullptr;            // on the preparing slot's stream: rows ready
    cudaEvent_t ev_use[RTS_STREAM_COUNT] = {};  // on each slot's stream: its contraction queued
    bool use_recorded[RTS_STREAM_COUNT] = {};
    // ... and their face sums computed while the Illum arrives: whole
    // directions copied by rts_send_illum_async in order from direction 0,
    // each summed on eager_st right after its copy
    cudaStream_t eager_st = nullptr;
    cudaEvent_t ev_sent = nullptr, ev_eager = nullptr;
    int64_t eager_next = -1;     // directions [0, eager_next) summed so far; -1: none
    int64_t eager_version = -1;  // inputs_version right after the last of those copies
    int eager_mode = -1;
};

// Device state of the transport sweep (rts_sweep.cu): the mesh, the
// per-direction structures of the local directions and the medium.  The unit
// of work is an out-face of a cell (its 3 nodes); per local direction d:
//   items[d]  out-faces in dependency order: cell << 8 | face << 6 | the
//             in-faces of its 3 nodes (2 bits each)
//   recs[d]   3 node distances per item (the LocX0 records' s, same order)
//   steps[d]  item offsets of the dependency steps (nsteps[d] + 1 entries)
//   bnd[d]    boundary in-faces, cell * 4 + face (nbnd[d] of them)
struct rts_sweep_state {
    int64_t N = 0, D = 0;            // cells, local directions
    std::vector<double> h_vert, h_normals;  // host copies for the builder
    std::vector<int32_t> h_pairs;
    double* d_vert = nullptr;        // [N][4][3]
    int32_t* d_pairs = nullptr;      // [N][4]
    double* d_normals = nullptr;     // [N][4][3]
    double* d_nodes = nullptr;       // [N][4][3][3] (MakeArrayX)
    uint32_t** d_items = nullptr;    // device pointer tables [D]
    double** d_recs = nullptr;
    int32_t** d_steps = nullptr;
    uint32_t** d_bnd = nullptr;
    int32_t* d_nsteps = nullptr;     // [D]
    int32_t* d_nbnd = nullptr;       // [D]
    std::vector<uint32_t*> h_items;  // host copies of the tables
    std::vector<double*> h_recs;
    std::vector<int32_t*> h_steps;
    std::vector<uint32_t*> h_bnd;
    std::vector<int32_t> h_nsteps, h_nbnd;
    std::vector<int64_t> h_nitems;
    std::vector<std::pair<void*, size_t>> blocks;  // allocations behind the tables
    std::vector<char> have;          // direction d built or imported
    double** d_att = nullptr;        // device pointer table [D] of the attenuation factors
    std::vector<double*> h_att;
    double* att_blk = nullptr;       // one factor per node record (exp(-k s), or a negative mark)
    size_t att_bytes = 0;
    bool att_valid = false;          // stored by a sweep since the last change of medium or structures
    double* d_med = nullptr;         // [N][4] k, beta, Q, 1/k (k = alpha + beta, or alpha)
    rts_medium md{};
    double bc[4] = {0.0, 0.0, 1.0, 0.0};
    bool has_medium = false;
    unsigned long long* d_norm = nullptr;  // norm bits + 1 (0: no term)
    int64_t records = 0, max_levels = 0;
};
void rts_sweep_free(rts_ctx* ctx);

struct rts_ctx {
    int device = 0;
    int num_sms = 0;
    int cc_major = 0, cc_minor = 0;
    cudaStream_t streams[RTS_STREAM_COUNT] = {nullptr, nullptr, nullptr};
    std::string last_error;

    int64_t budget_bytes = 0;
    int64_t used_bytes = 0;

    // directions (grid_directions_t)
    int64_t M = 0;
    double full_area = 0.0;
    std::vector<double> h_xyz, h_area;
    double* d_xyz = nullptr;   // [M][3]
    double* d_area = nullptr;  // [M]
    int phase = RTS_PHASE_THOMSON;
    double phase_g = 0.0;

    // grid
    int64_t N = 0;
    int64_t out_start = 0, out_end = 0;  // local out-directions (InitDevice start/end)
    double* d_illum = nullptr;   // [M][N][4]
    double* d_S = nullptr;       // [out_end-out_start][N]
    double* d_W = nullptr;       // [M][out_end-out_start]
    double* h_illum = nullptr;   // pinned, [M][N][4]
    double* h_S = nullptr;       // pinned, [out_end-out_start][N]
    double* d_energy = nullptr;  // [N]
    double* d_flux = nullptr;    // [N][3]
    double* d_geo = nullptr;     // [N][4][3] outward face normals, [N][4] face areas, [N] volumes (or null)
    double* d_params = nullptr;  // energy [N], flux [N][3], impuls [N][9], divstream [N], divimpuls [N][3]
    double* d_B = nullptr;       // [N]
    // residual bits (non-negative doubles order as u64): slot 0 for
    // rts_source_update, slots 1..RTS_RESID_CAP a ring of per-step residuals
    unsigned long long* d_resid = nullptr;
    unsigned long long* resid_target = nullptr;  // slot the next kernels reduce into
    int* d_flag = nullptr;       // device-side error flag of bounded waits
    cudaMemPool_t pool = nullptr;  // stream-ordered pool of the batched problems' buffers (created on first use)
    cudaStream_t serve_copy = nullptr;  // read-backs of finished serving requests
    cudaStream_t serve_admit = nullptr;  // set-up of admitted serving requests (lowest priority)

    // source iteration
    int solve_precision = -1;
    double solve_lambda = 0.0;
    bool solve_ready = false;
    bool solve_has_prev = false;
    int64_t solve_steps = 0;
    int call_precision = RTS_PREC_FP64;  // rts_scattering_async / rts_scattering (rts_set_precision)
    cudaEvent_t ev_order[RTS_STREAM_COUNT] = {};  // cross-stream ordering, one per waiting stream
    cudaEvent_t ev_inputs = nullptr;  // on the scattering stream: the device inputs of the integral calls written
    bool inputs_marked = false;       // ev_inputs covers every write of them queued so far
    int64_t inputs_version = 0;       // bumped at every write of the device Illum, W or scattering array
    cudaEvent_t ev_sync[RTS_STREAM_COUNT] = {};   // rts_sync_stream deadlines
    rts_split_state split;
    int split_flush = 0;         // hi*hi drain period in stages (0: default)
    int split_bias = 0;          // truncation correction: 0 conservation-based (relaxed steps), -1 none, >0 constant (1e-10 units)
    int tuning_epoch = 0;        // bumped when a setting that batch tables copy changes
    int64_t w_version = 0;       // bumped whenever d_W is rewritten
    int sweep_cache = 1;         // rts_sweep: store the attenuation factors once per medium (RTS_TUNE_SWEEP_CACHE)
    int serve_policy = 1;        // rts_serve_run: 0 all resident, 1 earliest deadline first, 2 least remaining work first
    int64_t serve_budget = 0;    // tiles per step for policy 1 (0: 8 waves of the SMs)
    int serve_slack = 500;       // policy 1 deadline: arrival + serve_slack / 100 x estimated isolated time
    std::vector<rts_tune_entry> tune;  // rts_autotune results, used for problems created with bn = 0
    rts_sweep_state* sweep = nullptr;  // transport sweep (rts_sweep_set_mesh)

    // instrumentation
    int64_t launches = 0;        // kernels launched by this context
    bool timing = false;         // record events around the dominant kernel
    std::vector<cudaEvent_t> tev;  // pairs (begin, end) of recorded launches
    size_t tev_used = 0;

    int64_t local() const { return out_end - out_start; }
};

// Event pair around the dominant kernel when timing is on (no-ops otherwise).
void rts_timing_begin(rts_ctx* ctx, cudaStream_t st);
void rts_timing_end(rts_ctx* ctx, cudaStream_t st);

// Device allocation accounted against the context's HBM budget.
int rts_dmalloc(rts_ctx* ctx, void** p, size_t bytes, const char* what);
void rts_dfree(rts_ctx* ctx, void* p, size_t bytes);
// Stream-ordered allocation from the context's pool (no device-wide
// synchronisation on either call; freed memory stays cached for reuse).
// Counted against the same HBM budget as rts_dmalloc.
int rts_pmalloc(rts_ctx* ctx, void** p, size_t bytes, const char* what, cudaStream_t st);
void rts_pfree(rts_ctx* ctx, void* p, size_t bytes, cudaStream_t st);

// Kernel launchers (defined in the .cu files).
int rts_launch_scatter_fp64(rts_ctx* ctx, int64_t k_begin, int64_t k_end, cudaStream_t st,
                            const double* B, double lambda, bool update, bool residual);
int rts_launch_moments(rts_ctx* ctx, cudaStream_t st);
int rts_launch_illum_params(rts_ctx* ctx, cudaStream_t st);
int rts_launch_update(rts_ctx* ctx, int64_t k_begin, int64_t k_end, cudaStream_t st,
                      const double* B, double lambda, bool residual);
int rts_launch_relax_fp64(rts_ctx* ctx, cudaStream_t st);
int rts_launch_weights(rts_ctx* ctx);
int rts_launch_synth(rts_ctx* ctx, uint64_t seed, double mu, double sigma, int independent_faces);

int rts_launch_weights_raw(rts_ctx* ctx, const double* d_xyz, const double* d_area, int M, int k_off, int loc,
                           double full_area, int phase, double g, double* W, cudaStream_t st);

// Operand preparation of the split-precision path (rts_prepass.cu).
// Split formats of the tensor-core operands: mode 0 BF16, 1 FP16 (scaled), 2 TF32.
// The device Illum, W or scattering array was (or is queued to be) written:
// the next integral call on another stream must wait for the write, and
// operands prepared from the old contents are stale.
inline void rts_inputs_written(rts_ctx* ctx)
{
    ctx->inputs_marked = false;
    ctx->inputs_version++;
}

// ... by a call other than the source iteration's own steps: the resident
// iteration must be set up again as well.
inline void rts_inputs_changed(rts_ctx* ctx)
{
    ctx->solve_ready = false;
    rts_inputs_written(ctx);
}

inline int rts_split_mode(int precision) { return precision == RTS_PREC_FP16X3 ? 1 : precision == RTS_PREC_TF32X3 ? 2 : 0; }
// extra (may be null): [Min] values of W^T row Mout (which must be < mpad)
int rts_pp_split_w(rts_ctx* ctx, const double* W, int Min, int Mout, int ldw, int kpad, int mpad, int mode,
                   uint16_t* Wc, float* cs, cudaStream_t st, const double* extra = nullptr);
// rs: per-row power-of-two scales putting 2 max(|Ibar|, |B|) into [2^13, 2^14)
// (and their inverses), computed in FP16 mode -- where the split applies them --
// and, with `bound`, in the other modes too, where they only bound the rows.
int rts_pp_rows_from_faces(rts_ctx* ctx, const double* illum, int64_t N, int64_t ld, int M, int kpad, const double* B, int mode,
                           float* rs, int64_t npad, uint16_t* A, cudaStream_t st, bool bound = false);
int rts_pp_rows_from_f32(rts_ctx* ctx, const float* ibar, int64_t N, int M, int64_t rows, int kpad, const float* B,
                         int mode, float* rs, int64_t rows_pad, uint16_t* A, cudaStream_t st, bool bound = false);
// The rows of rts_pp_rows_from_faces (bit for bit) in two passes that read the
// FP64 Illum once: FP64 face sums into the staging sums [M][N] with the
// per-cell max |face sum| into cmax [N] (the bits of a non-negative double),
// then the scales and the split from the staging; the FP64 pipe does only
// the 3 adds of each sum.
int rts_pp_rows_from_faces_staged(rts_ctx* ctx, const double* illum, int64_t N, int64_t ld, int M, int kpad,
                                  const double* B, int mode, float* rs, int64_t npad, uint16_t* A, double* sums,
                                  unsigned long long* cmax, cudaStream_t st, bool bound = false);
// Its two halves: the face sums of directions [j0, j1) (merging their maxima
// into cmax when non-null; cmax zeroed by the caller), and the scales and the
// split from the sums of all M directions.
int rts_pp_face_sums(rts_ctx* ctx, const double* illum, int64_t N, int64_t ld, int j0, int j1, double* sums,
                     unsigned long long* cmax, cudaStream_t st);
int rts_pp_rows_from_sums(rts_ctx* ctx, int64_t N, int M, int kpad, const double* B, int mode, float* rs, int64_t npad,
                          uint16_t* A, const double* sums, const unsigned long long* cmax, cudaStream_t st,
                          bool bound = false);
int rts_pp_join_rows(rts_ctx* ctx, const uint16_t* A, int64_t N, int M, int64_t rows, int kpad, const float* rs_inv,
                     int mode, double* out, cudaStream_t st);
int rts_pp_f32_to_f64(rts_ctx* ctx, const float* s, double* d, int64_t n, cudaStream_t st);
// Statistics of W (Mout == Min) for the conservation correction of relaxed
// steps, v [kpad + 4] FP32: v[j] = sum_k W[j][k] (FP64 sums) for j < Min, 0
// up to kpad; v[kpad] = 2^(7 - ceil(log2 sum_jk |W_jk|)) (the scale of the
// partial sums); v[kpad+1] c = the FP32 mean of the v_j; v[kpad+2] D = sum_j
// (v_j - c); v[kpad+3] = 1 / c.  u [Min] FP64: u_i = sum_j W[i][j] (v_j - c),
// the extra W^T row.  v64 [Min] FP64 scratch.
int rts_pp_w_stats(rts_ctx* ctx, const double* W, int Min, int Mout, int ldw, int kpad, float* v, double* v64,
                   double* u, cudaStream_t st);
int rts_pp_f64_to_f32(rts_ctx* ctx, const double* s, float* d, int64_t n, cudaStream_t st);

// Drain period (K-slices per FP32 drain) of the tensor-core path for a
// direction set, its out-direction columns [k0, k1) and phase kernel: 2 when
// W is smooth enough that the longer truncation chains stay far below the
// 1e-6 budget, else 1 (rts_flush.cpp).
int rts_auto_flush(const double* xyz, const double* area, int64_t M, double full_area, int64_t k0, int64_t k1,
                   int phase, double g, int precision);
// The context's drain period at a precision: RTS_TUNE_FLUSH when set, else
// rts_auto_flush of its directions, local out-directions and phase kernel.
int rts_ctx_flush(const rts_ctx* ctx, int precision);

// Tensor-core path (rts_split.cu).
// Autotuner tables (rts_tune.cpp).  Bucket of a problem's rows (cells x
// groups) in waves of 128-row tiles over the SMs: 0 below one wave, 1 below
// 4, 2 below 16, 3 from 16.
int rts_cells_bucket(const rts_ctx* ctx, int64_t rows);
// The drain period for a problem whose automatic period is `cap`: the tuned
// period with the shortest time among those allowed (1..cap for FP16 / BF16,
// cap itself for TF32), else cap.
int rts_tuned_flush(const rts_ctx* ctx, int64_t M, int precision, int64_t rows, int cap);
// The tuned tile width and order at that drain period; false if none.
bool rts_tuned_tile(const rts_ctx* ctx, int64_t M, int mode, int flush, int64_t rows, int* bn, int* order);
int rts_split_setup(rts_ctx* ctx, int precision);
int rts_split_step(rts_ctx* ctx, bool relax, cudaStream_t st);
// One evaluation from the device Illum (faces) into the FP64 device S, with
// the source update when B != nullptr; local out-directions [0, local).
int rts_split_host_call(rts_ctx* ctx, int precision, const double* illum_host, const double* B_host, double lambda,
                        double* S_host);
// One evaluation from the device Illum (faces) into the FP64 device S for
// every local out-direction, no host copies (the sweep's source iteration).
int rts_split_device_call(rts_ctx* ctx, int precision, cudaStream_t st);
// Local out-directions [start, end) from the device Illum (faces) into rows
// [start, end) of the FP64 device S on `st`, with the split operands of
// stream slot `slot` (no host copies, no host synchronisation once set up).
int rts_split_async(rts_ctx* ctx, int precision, int64_t start, int64_t end, int slot, cudaStream_t st);
// After a copy of [shift_dev, shift_dev + size) of the device Illum queued on
// the scattering stream at a tensor precision: the face sums of the directions
// it completes, on a stream of their own (rts_split.cu).
int rts_split_eager_send(rts_ctx* ctx, int64_t shift_dev, int64_t size);
int rts_split_read(rts_ctx* ctx, double* S_host);
int rts_split_read_ibar(rts_ctx* ctx, double* ibar_host);
void rts_split_free(rts_ctx* ctx);

// Bytes of one element of the given type, for accounting.
template <class T>
inline size_t rts_bytes(int64_t n) { return (size_t)n * sizeof(T); }
