// rts_group.h -- internal interface of the batched tensor-core path
// (rts_group.cu): resident problems and one-launch-per-step batches.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>

#include "rts_scatter.h"

struct rts_ctx;
struct rts_batch;

// One resident problem: split operands, scales, source, albedo, output.
struct GProb {
    int64_t id = 0;
    int64_t N = 0, M = 0, Mout = 0, groups = 1, rows = 0, rows_pad = 0, kpad = 0, mpad = 0;  // M: in-directions
    int bn = 0, n_tiles = 0, flush = 1;
    int order = 0;           // tile order of the kernel (GroupProblem::order)
    int64_t m_tiles = 0;
    bool fp16 = true;        // FP16 split with row / column scales (mode 1)
    int mode = 1;            // split mode: 0 BF16, 1 FP16, 2 TF32
    int64_t units = 0;       // 16-bit units per split row: 2*kpad, or 4*kpad for TF32
    uint16_t* wc = nullptr;  // [mpad][2*kpad] split W^T rows
    float* cs = nullptr;     // [2*mpad]: column scale, inverse
    uint16_t* a[2] = {nullptr, nullptr};  // [rows_pad][2*kpad] split Ibar rows (ping-pong)
    float* rs = nullptr;     // [2*rows_pad]: row scale, inverse
    bool a_ext = false;      // a[0] and rs belong to the caller (shared rows), not freed here
    float* B = nullptr;      // [rows]
    float* lam = nullptr;    // [groups]
    float* S32 = nullptr;    // [groups][Mout][N] (source iteration)
    double* S64 = nullptr;   // [groups][Mout][ldS] FP64 output (host-buffer calls), not owned
    int64_t ldS = 0;         // row pitch of the S output in cells (0: N)
    bool use_B = true;       // false: the bare integral (no source update)
    int cur = 0;
    int slot = -1;           // index of the problem's residual in the last launched table
    size_t bytes = 0;
    // energy-conservation correction of relaxed steps (iterative problems)
    float* vrow = nullptr;   // [kpad + 4] v_j = sum_k W[j][k]; then the quantum scale, c, D, 1/c (rts_pp_w_stats)
    void* part = nullptr;    // [n_tiles * 4][rows_pad] int4 per-slot partial sums of a step (fixed point)
    float* delta = nullptr;  // [rows_pad] per-row correction of the next step
    double* ex = nullptr;    // [rows_pad] sum_j v_j x_j of the current input (fixed-point quanta)
    alignas(64) unsigned char maps[3][128];
    alignas(64) unsigned char rmaps[2][128];  // relaxation boxes of a[0], a[1]
};

void rts_group_geometry(int64_t Min, int64_t Mout, int64_t rows, int bn_override, int* bn, int* n_tiles, int64_t* kpad,
                        int64_t* mpad, int64_t* rows_pad, int64_t* m_tiles);
int64_t rts_group_footprint(int64_t N, int64_t M, int64_t groups, bool iterative, int mode = 1);
int rts_group_batch_new(rts_ctx* ctx, rts_batch** out);
void rts_group_batch_free(rts_batch* b);
// buffers allocated and initialised on st (null: the scattering stream)
// ext_a / ext_rs (single evaluations only): split Ibar rows and row scales the
// caller owns and fills, laid out as this problem's own would be
int rts_group_new_problem(rts_batch* b, int64_t N, int64_t Min, int64_t Mout, int64_t groups, const double* W_dev, int ldw,
                          int mode, int flush, int bn_override, bool iterative, GProb** out, cudaStream_t st = nullptr,
                          uint16_t* ext_a = nullptr, float* ext_rs = nullptr);
// W (and, for problems with the correction, its statistics and extra row)
// into the problem's split W^T rows, on st.
int rts_group_set_w(rts_ctx* ctx, GProb* p, const double* W_dev, int ldw, cudaStream_t st);
int rts_group_attach(rts_batch* b, GProb* p, int64_t* id);
GProb* rts_group_find(rts_batch* b, int64_t id, size_t* index);
int rts_group_remove(rts_batch* b, int64_t id);
int rts_group_remove_on(rts_batch* b, int64_t id, cudaStream_t st);
int rts_batch_add_on(rts_batch* batch, const rts_problem_desc* d, const float* ibar, const float* B,
                     const double* lambda, cudaStream_t st, bool sync, int64_t* id);
int rts_group_step(rts_batch* b, int relax, cudaStream_t st);
// Builds and uploads the device table now (a later step of an unchanged batch
// then queues its launch without a host synchronisation).
int rts_group_prepare(rts_batch* b, int relax, cudaStream_t st);
int rts_group_step_subset(rts_batch* b, int relax, const int64_t* ids, int n, cudaStream_t st);
int rts_group_step_pieces(rts_batch* b, int relax, const int64_t* ids, const int64_t* first, const int64_t* count,
                          int n, cudaStream_t st);
int64_t rts_group_problem_tiles(rts_batch* b, int64_t id);
int rts_group_capture(rts_batch* b, int steps, int relax);
int rts_group_replay(rts_batch* b);
int64_t rts_group_total_tiles(rts_batch* b);
size_t rts_group_count(rts_batch* b);
unsigned long long* rts_group_resid_slot(rts_batch* b, size_t index);
// st: stream the scratch and direction buffers are used on (null: the scattering stream)
int rts_group_scratch(rts_batch* b, size_t bytes, void** p, cudaStream_t st = nullptr);
int rts_group_dirs(rts_batch* b, const double* xyz, const double* area, int64_t M, double** d_xyz,
                   double** d_area, cudaStream_t st = nullptr);
rts_ctx* rts_group_ctx(rts_batch* b);
// Forces the device table to be rebuilt before the next launch (after the
// caller changed cur / S64 / use_B of a problem) and drops a captured graph.
void rts_group_invalidate(rts_batch* b);
float rts_group_bias(const rts_ctx* ctx, int mode, int flush);
// Bytes of the energy-correction buffers of an iterative problem.
int64_t rts_group_energy_bytes(int64_t kpad, int64_t rows_pad, int n_tiles);
// Clears the per-row corrections (a restarted iteration starts uncorrected)
// and computes sum_j v_j x_j of the current split input: after the rows of
// the problem's input were written.
int rts_group_reset_energy(rts_ctx* ctx, GProb* p, cudaStream_t st);
