/*
 * rts_scatter.h -- C ABI of the GB300 scattering-integral library
 * (librts_scatter.so).
 *
 * The library computes the scattering integral of the radiation-transport
 * source iteration of relativistic_solver_hllc,
 *
 *     S[k][c] = sum_j W[j][k] * Ibar[j][c],   Ibar[j][c] = (1/4) sum_f Illum[j][c][f]
 *     W[j][k] = Gamma(w_j, w_k) * area_j / full_area      (Thomson, reference form)
 *
 * followed (optionally) by the source update S <- (1-lambda) B + lambda S,
 * plus the FP64 direction moments (energy, flux) and the FP64 convergence
 * residual.  Data layouts are the reference's: Illum is [direction][cell][face]
 * FP64 (grid_t::Illum, solve_module/solve_global_struct.h:153-230) and the
 * scattering array is [local out-direction][cell] FP64 (grid_t::scattering).
 *
 * Every entry point returns an rts_status; none calls exit().  Sizes and
 * offsets are 64-bit.  A context is used by one host thread at a time.
 * Reference paths below are relative to solver_hllc_illum_cuda/.
 */
#ifndef RTS_SCATTER_H
#define RTS_SCATTER_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTS_ABI_VERSION 1

typedef enum rts_status {
    RTS_OK = 0,
    RTS_ERR_INVALID_ARGUMENT = 1, /* bad size, null pointer, range outside the grid */
    RTS_ERR_CUDA = 2,             /* a CUDA runtime call or launch failed */
    RTS_ERR_OUT_OF_MEMORY = 3,    /* device or pinned host allocation failed */
    RTS_ERR_BAD_STATE = 4,        /* call out of order (e.g. scatter before init) */
    RTS_ERR_TIMEOUT = 5,          /* a host-side wait reached its deadline */
    RTS_ERR_OVER_BUDGET = 6,      /* allocation refused by the HBM budget */
    RTS_ERR_UNSUPPORTED = 7,      /* mode not built for this device / size */
    RTS_ERR_DEVICE_WAIT = 8       /* a bounded device-side wait gave up */
} rts_status;

/* Stream slots: e_cuda_stream_id_t (solve_module/solve_global_struct.h:234-240),
 * created with the same priorities as SetDevice (cuda/cuda_solve.cu:46-67). */
typedef enum rts_stream_id {
    RTS_STREAM_SCATTERING_1 = 0,
    RTS_STREAM_SCATTERING_2 = 1,
    RTS_STREAM_PARAMS = 2,
    RTS_STREAM_COUNT = 3
} rts_stream_id;

/* Direction-pair kernels. */
typedef enum rts_phase {
    RTS_PHASE_THOMSON = 0, /* Gamma = 3(1+mu^2)/4, W = Gamma*area_j/full_area (cuda/cuda_utils.cu:7-16) */
    RTS_PHASE_HG = 1,      /* Henyey-Greenstein, each out-direction column renormalised to sum 1 */
    RTS_PHASE_CUSTOM = 2   /* W supplied by the caller (rts_set_weights) */
} rts_phase;

/* Arithmetic of the contraction. */
typedef enum rts_precision {
    RTS_PREC_FP64 = 0,   /* FP64 CUDA cores; matches the CPU integral to 1e-12 relative */
    RTS_PREC_BF16X3 = 1, /* tcgen05 tensor cores, split BF16 hi/lo, three products, FP32 accumulate */
    RTS_PREC_FP16X3 = 2, /* tcgen05 tensor cores, scaled split FP16 hi/lo, three products, FP32 accumulate */
    RTS_PREC_TF32X3 = 3  /* tcgen05 tensor cores (kind::tf32), split TF32 hi/lo, three products, FP32
                            accumulate: no scaling, FP32 range, half the FP16 path's tensor rate */
} rts_precision;

typedef struct rts_ctx rts_ctx;

/* ---------------------------------------------------------------------- */
/* context, devices, streams                                               */
/* ---------------------------------------------------------------------- */

int rts_abi_version(void);

/* Replaces SetDevice (cuda/cuda_solve.cu:46-67): selects the device and
 * creates the three priority streams. */
int rts_ctx_create(int device, rts_ctx** out);

/* Replaces ClearDevice + ClearHost (cuda/cuda_struct.cu:180-214): frees every
 * device and pinned host buffer of the context.  Accepts NULL. */
int rts_ctx_destroy(rts_ctx* ctx);

/* Text of the last error raised on this context ("" if none). */
const char* rts_last_error(const rts_ctx* ctx);

/* Cap on the device bytes this context may hold (default: 90% of the
 * device memory free at creation).  Allocations beyond it fail with
 * RTS_ERR_OVER_BUDGET. */
int rts_set_hbm_budget(rts_ctx* ctx, int64_t bytes);
int rts_hbm_used(const rts_ctx* ctx, int64_t* bytes);

/* ---------------------------------------------------------------------- */
/* grid and directions                                                     */
/* ---------------------------------------------------------------------- */

/* Replaces InitDevice (cuda/cuda_struct.cu:134-178,187-190) for the
 * scattering path.  Directions: xyz [M][3], area [M], full_area
 * (grid_directions_t, global_def.h:79-90).  Allocates device Illum
 * [M][N][4], device scattering [end-start][N] for the local out-directions
 * [start, end), and the pinned host Illum / scattering arrays that InitDevice
 * hands to grid_t (cuda/cuda_struct.cu:154-156).  The phase kernel defaults
 * to RTS_PHASE_THOMSON. */
int rts_init(rts_ctx* ctx, const double* xyz, const double* area, int64_t M, double full_area,
             int64_t N, int64_t start, int64_t end);

/* Pinned host arrays owned by the context (grid_t::Illum, grid_t::scattering). */
int rts_host_illum(rts_ctx* ctx, double** illum);
int rts_host_scattering(rts_ctx* ctx, double** scattering);

/* Phase kernel for later integrals (recomputes the FP64 W). */
int rts_set_phase(rts_ctx* ctx, int phase, double g);

/* Caller-supplied W[j][k] for j in [0, M), k in the local out-directions
 * (row-major, (end-start) columns).  Sets the phase to RTS_PHASE_CUSTOM. */
int rts_set_weights(rts_ctx* ctx, const double* W);

/* ---------------------------------------------------------------------- */
/* Illum transfer                                                          */
/* ---------------------------------------------------------------------- */

/* Replaces CudaSendIllumAsync(size, shift_dev, shift_host, Illum_host)
 * (cuda/cuda_solve.cu:77-83) and, with shift_dev == shift_host, the
 * two-argument overload (:69-76).  Counts are in doubles; the copy goes on
 * stream RTS_STREAM_SCATTERING_1 as in the reference (cuda_streams[0]). */
int rts_send_illum_async(rts_ctx* ctx, int64_t size, int64_t shift_dev, int64_t shift_host,
                         const double* illum_host);

/* Replaces CopyIllumOnDevice (cuda/cuda_solve.cu:85-88): synchronous copy of
 * the first `size` doubles. */
int rts_copy_illum(rts_ctx* ctx, int64_t size, const double* illum_host);

/* ---------------------------------------------------------------------- */
/* scattering integral (FP64, the drop-in path)                            */
/* ---------------------------------------------------------------------- */

/* Arithmetic of the reference-compatible integral calls rts_scattering_async
 * and rts_scattering (rts_precision; RTS_PREC_FP64 by default, which matches
 * the reference's CPU integral to 1e-12 relative).  A tensor precision runs
 * the same calls on the tcgen05 split path (RTS_PREC_FP16X3 and
 * RTS_PREC_TF32X3 to 1e-6 relative, RTS_PREC_BF16X3 to ~1e-5): the
 * reference's kernel d_GetS_MPI_Stream at that precision, behind the same
 * call.  RTS_ERR_UNSUPPORTED for a tensor precision on a device other than
 * sm_10x.  At a tensor precision the calls also hold the split Ibar rows
 * (4 bytes per cell and in-direction, 8 for RTS_PREC_TF32X3) and, where the
 * HBM budget and the device leave room, a staging of the FP64 face sums
 * (8 bytes per cell and direction) that speeds up their preparation; without
 * that room the rows are prepared directly, with the same results. */
int rts_set_precision(rts_ctx* ctx, int precision);
int rts_get_precision(const rts_ctx* ctx, int* precision);

/* Replaces CalculateIntScatteringAsyncMPIStream (cuda/cuda_solve.cu:89-111,
 * kernel d_GetS_MPI_Stream at cuda/cuda_kernel.cu:82-111): computes local
 * out-directions [start, end) of the device Illum on `stream`, at the
 * context's precision (rts_set_precision), and queues the D2H of rows
 * [start, end) to host_out + start*N (host_out NULL: the pinned host
 * scattering array).  The reference offsets the copy by `start` elements,
 * which is right only for start == 0; this entry point uses start*N.  Work on
 * a stream other than RTS_STREAM_SCATTERING_1 is ordered after the writes of
 * the device Illum, W and scattering array queued there (the Illum copies of
 * rts_send_illum_async among them), not after the integral calls queued
 * there: calls on different streams overlap, as the reference's pair on
 * scattering streams 1 and 2 does (solve_module/illum/Illum_async.cpp:
 * 1019-1020).  At a tensor precision each stream slot has split operands of
 * its own, and rows both calls cover receive the same values from either.
 * As in the reference, Illum copies queued after a call on another stream
 * are not ordered after that call: synchronise the streams
 * (rts_sync_stream) before rewriting the Illum. */
int rts_scattering_async(rts_ctx* ctx, int64_t start, int64_t end, int stream, double* host_out);

/* Replaces CalculateIntScattering (cuda/cuda_solve.cu:153-170): copies
 * illum_host (all M*N*4 doubles; NULL: the pinned host Illum) to the device,
 * computes every local out-direction at the context's precision and copies
 * the result to host_out (NULL: the pinned host scattering array),
 * synchronously. */
int rts_scattering(rts_ctx* ctx, const double* illum_host, double* host_out);

/* Copies rows [start, end) of the device scattering array to host_out +
 * start*N on `stream` without recomputing them (the D2H half of
 * CalculateIntScatteringAsyncMPIStream, cuda/cuda_solve.cu:107-108). */
int rts_read_scattering(rts_ctx* ctx, int64_t start, int64_t end, int stream, double* host_out);

/* One evaluation with host buffers at the given precision (rts_precision):
 * copies illum_host (M*N*4 doubles, reference layout) and B_host (N values)
 * to the device, computes S = (1-lambda) B + lambda W^T Ibar for every local
 * out-direction and copies S (FP64, [local][N]) to S_host, synchronously.
 * With lambda = 1 and B ignored this is CalculateIntScattering at the
 * requested precision. */
int rts_scattering_update(rts_ctx* ctx, int precision, const double* illum_host,
                          const double* B_host, double lambda, double* S_host);

/* Copies rows [start, end) of a host scattering array (host + start*N) into
 * the device scattering array on `stream`, the H2D counterpart of
 * rts_read_scattering: the source term of the device sweep when the
 * scattering comes from elsewhere (the reference's CPU sweep reads
 * grid_t::scattering from host memory). */
int rts_send_scattering(rts_ctx* ctx, int64_t start, int64_t end, int stream, const double* host);

/* Allocation-free FP64 scattering integral.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory --
 * code that runs inside a caller-owned memory pool or arena that forbids
 * allocations outside it, and hosts that budget every device byte up front.
 * The caller passes device pointers: Illum [M][N][4] (16-byte aligned: it is
 * read as pairs of doubles), directions xyz [M][3] and area [M], and the
 * output scattering [M][N] (all out-directions), the last three 8-byte
 * aligned; a misaligned pointer returns RTS_ERR_INVALID_ARGUMENT before
 * anything is launched.  The work is queued on `stream` (a cudaStream_t, NULL
 * for the default stream) and nothing is synchronised or allocated -- no
 * cudaMalloc, cudaFree or allocating library call.  The only scratch, the
 * M x M FP64 direction-pair matrix, lives in a fixed 2 MB device array of the
 * library that every GPU loading the library holds until the process exits;
 * hence the limit M <= RTS_NOALLOC_MAX_DIRS (larger M returns
 * RTS_ERR_INVALID_ARGUMENT).  The scratch is shared by all calls and
 * rewritten in full by each: calls that overlap on the GPU race.  Each call
 * outside a stream capture looks the scratch address up for the current
 * device (cudaGetSymbolAddress); a call made while its stream is being
 * captured reuses the address of the last uncaptured call on that device, so
 * make the first call on a device before any stream capture.  An error that
 * the caller's own earlier work left pending is returned as RTS_ERR_CUDA
 * without launching and is left pending. */
#define RTS_NOALLOC_MAX_DIRS 512
int rts_scattering_noalloc(const double* d_illum, const double* d_xyz, const double* d_area, int64_t N,
                           int64_t M, double full_area, double* d_scattering, void* stream);

/* Device pointers of the resident arrays (for callers that keep data on the
 * GPU): Illum [M][N][4] and scattering [end-start][N]. */
int rts_device_arrays(rts_ctx* ctx, double** d_illum, double** d_scattering);

/* ---------------------------------------------------------------------- */
/* moments, update, residual                                               */
/* ---------------------------------------------------------------------- */

/* Energy E[c] = sum_j Ibar*area_j/full_area and flux F[c][3] =
 * sum_j w_j Ibar*area_j/full_area in FP64 (cuda/cuda_utils.cu:18-67,
 * cuda/cuda_kernel.cu:113-134), on `stream`; results copied to the host
 * arrays that are non-NULL, synchronously with that stream. */
int rts_moments(rts_ctx* ctx, int stream, double* energy, double* flux);

/* Cell geometry for the divergence moments: outward unit normals of the four
 * faces [N][4][3], face areas [N][4], cell volumes [N] (> 0).  Replaces the
 * reference's reads of normals.bin / squares.bin / volume.bin in InitDevice
 * and their upload (cuda/cuda_struct.cu:134-176, grid_init_copy_host_to_device
 * :86-107). */
int rts_set_geometry(rts_ctx* ctx, const double* normals, const double* face_areas, const double* volume);

/* Energy [N], flux [N][3], impulse tensor [N][9] (row-major, symmetric), and
 * the divergences of flux [N] and impulse [N][3] of the device Illum, in FP64,
 * in one pass.  Replaces d_MakeIllumParam and its launches
 * CalculateAllParam / CalculateAllParamStream (cuda/cuda_kernel.cu:218-223,
 * cuda/cuda_solve.cu:272-320), CalculateImpuls (:209-225), CalculateDivImpuls
 * (:227-247) and CalculateDivStream (:249-270).  Null outputs are skipped; the
 * divergences need rts_set_geometry.  Runs on `stream` after the work queued
 * on the scattering stream and returns when the copies have landed. */
int rts_illum_params(rts_ctx* ctx, int stream, double* energy, double* flux, double* impuls, double* divstream,
                     double* divimpuls);

/* S <- (1-lambda) B[c] + lambda S on the device scattering array
 * (local rows [start, end)), and the FP64 residual max|S_new - S_old|
 * against the values it replaces (residual may be NULL). */
int rts_source_update(rts_ctx* ctx, const double* B_host, double lambda, int64_t start,
                      int64_t end, int stream, double* residual);

/* ---------------------------------------------------------------------- */
/* synchronisation                                                         */
/* ---------------------------------------------------------------------- */

/* Replaces CudaSyncStream (cuda/cuda_solve.cu:37-40) with a deadline:
 * timeout_us < 0 waits without limit, otherwise RTS_ERR_TIMEOUT when the
 * stream's work has not finished in time (the work keeps running). */
int rts_sync_stream(rts_ctx* ctx, int stream, int64_t timeout_us);

/* Replaces CudaWait (cuda/cuda_solve.cu:42-45) with a deadline. */
int rts_wait(rts_ctx* ctx, int64_t timeout_us);

/* ---------------------------------------------------------------------- */
/* device-resident source iteration                                        */
/* ---------------------------------------------------------------------- */

/* Prepares a source iteration on the Illum already on the device:
 * precision (rts_precision), source B [N] (host, FP64), albedo lambda.
 * Requires the local out-directions to be all M directions.  For the tensor
 * precisions this builds the split operands of W and Ibar on the device. */
int rts_solve_setup(rts_ctx* ctx, int precision, const double* B_host, double lambda);

/* One evaluation: S_int = W^T Ibar, S = (1-lambda) B + lambda S_int,
 * residual = max|S - S_prev| (FP64, S_prev = 0 before the first step); then,
 * if relax != 0, Ibar <- 0.5 Ibar + 0.5 S for the next step.  All on
 * RTS_STREAM_SCATTERING_1; *residual (may be NULL) is read back, which
 * synchronises the stream. */
int rts_solve_step(rts_ctx* ctx, int relax, double* residual);

/* Same step with nothing read back (for timing loops); the residual of the
 * step stays on the device and rts_solve_residual fetches it. */
int rts_solve_step_async(rts_ctx* ctx, int relax);
int rts_solve_residual(rts_ctx* ctx, double* residual);

/* Residuals of the last n steps since rts_solve_setup, oldest first
 * (n <= 4096). */
int rts_solve_residual_history(rts_ctx* ctx, double* out, int64_t n);

/* Copies the current S [M][N] (FP64) to the host. */
int rts_solve_read(rts_ctx* ctx, double* S_host);

/* Copies the first `size` doubles of the device Illum to the host (the
 * reverse of rts_copy_illum), synchronously. */
int rts_read_illum(rts_ctx* ctx, int64_t size, double* illum_host);

/* Copies the current face-mean intensity Ibar [M][N] (FP64) to the host. */
int rts_solve_read_ibar(rts_ctx* ctx, double* ibar_host);

/* ---------------------------------------------------------------------- */
/* batched problems: one persistent tensor-core launch per step            */
/* ---------------------------------------------------------------------- */
/* Many independent scattering problems (own cell count, direction set,
 * phase kernel, precision, frequency groups, albedo) are kept resident and
 * advanced together: every step is one launch of the grouped tcgen05 kernel
 * over the tiles of all problems (source update, residual and relaxation
 * fused), and a fixed number of steps can be captured into a CUDA graph and
 * replayed.  No counterpart in the reference, which solves one problem per
 * process. */
typedef struct rts_batch rts_batch;

typedef struct rts_problem_desc {
    int64_t N;      /* cells per frequency group */
    int64_t M;      /* directions: spherical Fibonacci set of M points, weights 4 pi / M */
    int64_t groups; /* frequency groups sharing the direction set and phase kernel (>= 1) */
    int phase;      /* RTS_PHASE_THOMSON or RTS_PHASE_HG */
    double g;       /* Henyey-Greenstein asymmetry, (-1, 1) */
    int precision;  /* RTS_PREC_FP16X3 or RTS_PREC_BF16X3 */
    int flush;      /* K-slices per FP32 drain (1 or 2; 0: automatic, see RTS_TUNE_FLUSH) */
    int bn;         /* out-directions per tile, multiple of 16, <= 256 (0: balanced default) */
} rts_problem_desc;

/* Device bytes a problem holds while resident (for admission control). */
int rts_problem_footprint(const rts_problem_desc* desc, int64_t* bytes);

int rts_batch_create(rts_ctx* ctx, rts_batch** out);
int rts_batch_destroy(rts_batch* batch);

/* Adds a problem.  ibar: host [groups][M][N] FP32 face-mean intensity
 * (direction-major, as grid_t::scattering); B: host [groups][N] FP32 source;
 * lambda: host [groups] albedo.  The copies complete before the call returns. */
int rts_batch_add(rts_batch* batch, const rts_problem_desc* desc, const float* ibar, const float* B,
                  const double* lambda, int64_t* id);
int rts_batch_remove(rts_batch* batch, int64_t id);
int rts_batch_size(rts_batch* batch, int64_t* problems, int64_t* tiles);

/* One step of every problem (relax != 0: Ibar <- 0.5 Ibar + 0.5 S after it). */
int rts_batch_step(rts_batch* batch, int relax);

/* Captures `steps` steps into a CUDA graph (invalidated by add / remove) and
 * replays it. */
int rts_batch_capture(rts_batch* batch, int steps, int relax);
int rts_batch_replay(rts_batch* batch);

/* Waits for the batch's work with a deadline (timeout_us < 0: no limit). */
int rts_batch_sync(rts_batch* batch, int64_t timeout_us);

/* S [groups][M][N] FP32 of a problem (host), and the FP64 residual
 * max|S - S_prev| of its last step (either may be NULL); synchronous. */
int rts_batch_read(rts_batch* batch, int64_t id, float* S, double* residual);

/* ---------------------------------------------------------------------- */
/* serving: continuous batching of scattering solves                       */
/* ---------------------------------------------------------------------- */
typedef struct rts_request {
    double arrival_s;       /* arrival, seconds after the start of the run (non-decreasing) */
    rts_problem_desc desc;  /* the problem */
    int iterations;         /* source iterations to run (relaxation after each) */
    const float* ibar;      /* host [groups][M][N] FP32 initial face-mean intensity */
    const float* B;         /* host [groups][N] FP32 source */
    const double* lambda;   /* host [groups] albedo */
    float* S_out;           /* host [groups][M][N] result, or NULL */
} rts_request;

typedef struct rts_serve_stats {
    int64_t completed, rejected, max_active, steps, peak_bytes;
    double makespan_s;
    double throughput;      /* cell-direction-iterations per second */
    double p50_ms, p99_ms, mean_ms, max_ms;
    double admit_s, step_s, retire_s;  /* host time in admission (set-up), device steps, retirement */
} rts_serve_stats;

/* Runs the requests through one device batch with continuous batching:
 * arrived requests are admitted in arrival order while the context's device
 * bytes stay under hbm_cap, every step advances all resident requests by one
 * iteration in one grouped launch, finished requests are read back and leave.
 * latency_ms[i] (may be NULL) receives request i's latency, -1 if rejected.
 * step_timeout_us bounds every device wait.  No counterpart in the reference. */
int rts_serve_run(rts_ctx* ctx, const rts_request* reqs, int64_t n, int64_t hbm_cap, int64_t step_timeout_us,
                  double* latency_ms, rts_serve_stats* stats);

/* Pinned host memory (for request inputs and results). */
int rts_host_alloc(int64_t bytes, void** ptr);
int rts_host_free(void* ptr);

/* ---------------------------------------------------------------------- */
/* synthetic inputs (benchmark workloads; not part of the reference API)   */
/* ---------------------------------------------------------------------- */

/* Fills the device Illum with lognormal(mu, sigma) values from the same
 * counter hash as the CPU generator (stream 1, index j*N+c, or
 * (j*N+c)*4+f with independent_faces). */
int rts_synth_illum(rts_ctx* ctx, uint64_t seed, double mu, double sigma, int independent_faces);

/* Adds a batched problem whose inputs are generated on the device from the
 * counter hash: Ibar [g][j][c] lognormal(mu, sigma) (stream 1, index
 * (g*M + j)*N + c), B [g][c] uniform(b_lo, b_hi) (stream 2, index g*N + c). */
int rts_batch_add_synthetic(rts_batch* batch, const rts_problem_desc* desc, uint64_t seed, double mu, double sigma,
                            double b_lo, double b_hi, const double* lambda, int64_t* id);

/* n values of the counter hash (stream, indices i0..i0+n) generated on the
 * device and copied to host memory: lognormal(a, b) if lognormal != 0, else
 * uniform(a, b). */
int rts_synth_host_f32(rts_ctx* ctx, uint64_t seed, uint64_t stream, int lognormal, double a, double b, int64_t i0,
                       int64_t n, float* host_out);

/* Spherical Fibonacci direction set: xyz [M][3], area [M] = 4 pi / M,
 * full_area = 4 pi (host only, no context needed). */
int rts_synth_directions(int64_t M, double* xyz, double* area, double* full_area);

/* uniform(lo, hi) values of counter-hash stream `stream`, indices
 * [i0, i0 + n) (host only). */
int rts_synth_uniform(uint64_t seed, uint64_t stream, double lo, double hi, int64_t i0, int64_t n,
                      double* out);

/* ---------------------------------------------------------------------- */
/* host formats and partition (no GPU involved)                            */
/* ---------------------------------------------------------------------- */

/* Direction-set text file of ReadSphereDirectionDecartToSpherical
 * (file_module/reader_txt.cpp:25-47): M, then M lines "area x y z", then
 * full_area.  With xyz or area NULL, or capacity < M, only *M is returned. */
int rts_read_direction_file(const char* path, int64_t capacity, int64_t* M, double* xyz, double* area,
                            double* full_area);
int rts_write_direction_file(const char* path, int64_t M, const double* xyz, const double* area,
                             double full_area);

/* Count-prefixed binary arrays of ReadSimpleFileBin / WriteSimpleFileBin
 * (file_module/reader_bin.h:13-30, file_module/writer_bin.h:9-26): int32
 * count, then the raw elements.  With data NULL or capacity < count, only
 * *count is returned. */
int rts_read_simple_bin(const char* path, int64_t elem_size, int64_t capacity, void* data, int64_t* count);
int rts_write_simple_bin(const char* path, int64_t elem_size, int64_t count, const void* data);

/* The radiation part of the solution dump WriteFileSolution
 * (file_module/writer_bin.cpp:15-44, CUDA build) from the device state, into
 * directory dir: Illum.bin (face mean of direction 0 per cell), energy.bin,
 * stream.bin, impuls.bin and, when rts_set_geometry was called, divstream.bin
 * and divimpuls.bin, each an int32 count then the raw FP64 elements. */
int rts_write_solution(rts_ctx* ctx, const char* dir);

/* Out-direction partition over np ranks: GetSend / GetDisp
 * (solve_module/solve_utils.cpp:177-202). */
int rts_partition(int np, int64_t n, int64_t* send, int64_t* disp);

/* ---------------------------------------------------------------------- */
/* transport sweep: the producer of Illum                                  */
/* ---------------------------------------------------------------------- */

/* Codes of a face without a neighbour in the pairs array (eBoundaryTypes,
 * global_def.h:45-51). */
#define RTS_BOUND_FREE (-1)
#define RTS_BOUND_LOCK (-2)
#define RTS_BOUND_OUTSOURCE (-3)
#define RTS_BOUND_INNER (-4)

/* The medium of GetCurIllum (solve_module/illum/Illum_async.cpp:259-470).
 * RTS_MEDIUM_SCATTERING, classes 0, 1, 3, 10 and 11:
 *     k = alpha + beta, ss = s * s_scale, S' = S * i_scale, I0' = I0 * i_scale,
 *     I = exp(-k ss) (I0' k + (exp(k ss) - 1)(Q + S' beta)) / k     (k > 1e-10)
 *     I = (1 - ss k)(I0' + ss (Q + S' beta))                       (otherwise)
 *     result max(I, 0) / i_scale;
 * RTS_MEDIUM_ABSORPTION, class 2:
 *     I = I0 exp(-alpha ss) + Q (1 - exp(-alpha ss)) / alpha        (alpha > 1e-15)
 *     I = I0 (1 - alpha ss) + Q ss                                  (otherwise)
 *     result max(I, 0).
 * alpha, beta, Q are per cell; s_scale is 1 (DIST for class 11, 388189e5 for
 * class 2) and i_scale 1 (RADIATION for class 11).  With radius > 0 the
 * ball_* coefficients hold at the nodes inside the ball (class 0's source
 * region). */
#define RTS_MEDIUM_SCATTERING 0
#define RTS_MEDIUM_ABSORPTION 1
typedef struct rts_medium {
    int mode;
    int reserved;
    double s_scale;
    double i_scale;
    double ball[3];
    double radius;
    double ball_alpha, ball_beta, ball_q;
} rts_medium;

/* Synthetic mesh (host only, no device work): the unit cube cut into n^3
 * hexahedra (x fastest), each cut into 6 tetrahedra around its diagonal from
 * (0,0,0) to (1,1,1); N = 6 n^3 cells.  vert [N][4][3]; pairs [N][4] the
 * neighbour's cell*4 + face or a boundary code; normals [N][4][3] outward
 * unit normals, face f opposite vertex {2,0,1,3}[f] (VTK's tetra faces
 * {0,1,3}, {1,2,3}, {2,0,3}, {0,2,1}).  bound_rule 0: every boundary face
 * RTS_BOUND_FREE (the reference's Cube variant of SetTypeOfBound,
 * utils/grid_geometry/geometry_data.cpp:512-517); 1: faces of the x = 0 side
 * RTS_BOUND_OUTSOURCE, of the x = 1 side RTS_BOUND_FREE, others
 * RTS_BOUND_LOCK (its Cone variant, :484-504).  tilt != 0 turns the cube about
 * its centre by a fixed rotation (Rx 0.3, Ry 0.2, Rz 0.1 rad; boundary codes
 * from the unturned faces) so that no face is parallel to a
 * spherical-Fibonacci direction.  n in [1, 127]. */
int rts_mesh_cube(int n, int bound_rule, int tilt, double* vert, int32_t* pairs, double* normals);

/* The mesh of the sweep for the context's N cells (rts_init): vertices
 * [N][4][3] (vertex.bin), pairs [N][4] (pairs.bin) and outward unit face
 * normals [N][4][3] (normals.bin), the inputs that make_illum_struct and
 * build_graph read (make_illum_struct/struct_short_characteristics_main.cpp:
 * 28-74).  Copied to the device; the per-direction structures are dropped. */
int rts_sweep_set_mesh(rts_ctx* ctx, const double* vert, const int32_t* pairs, const double* normals);

/* Builds the per-direction structures of the local directions on the
 * device, the work of make_illum_struct and build_graph: the in/out state of
 * every face (GetInAndOutFaces, utils/grid_geometry/geometry_solve.cpp:212-227),
 * the cells in dependency order (build_graph_calculation.cpp:347-510: steps
 * of cells whose in-faces are all known, each step in ascending cell id),
 * and for every out-face node (MakeArrayX) the in-face hit going back along
 * the direction and the distance to it (CalculateNodeValue,
 * struct_short_characteristics_logic_function.cpp:222-254).  *records (may
 * be NULL) receives the node count over all local directions, *levels the
 * largest number of steps of one direction.  RTS_ERR_UNSUPPORTED when a
 * direction's dependencies form a cycle or a node finds no in-face (a
 * direction parallel to a face). */
int rts_sweep_build(rts_ctx* ctx, int64_t* records, int64_t* levels);

/* The same structures from the reference's make_illum_struct / build_graph
 * files of local direction d: order [N] (graph<d>.bin), states [N]
 * (state_face<d>.bin, bit f set for an in-face) and the LocX0<d>.bin records
 * (cell_local, global_def.h:101-108: FP64 s at byte 0, uint8 in-face id at
 * byte 24, 32-byte stride), `count` of them in the file's order.  Every
 * local direction must be imported (or rts_sweep_build called) before
 * rts_sweep. */
int rts_sweep_import_direction(rts_ctx* ctx, int64_t d, const int32_t* order, const int32_t* states,
                               const void* locx0, int64_t count);

/* The structures of local direction d in the reference's file layouts: order
 * [N] (graph<d>.bin: cells in dependency order), states [N] (state_face<d>.bin)
 * and, when capacity >= *count, the LocX0<d>.bin records (32 bytes each: FP64 s,
 * the 2-D x0 left zero -- the sweep does not read it -- and the uint8 in-face
 * id at byte 24) in the order of `order`.  Any output may be NULL; *count
 * receives the record count. */
int rts_sweep_export_direction(rts_ctx* ctx, int64_t d, int32_t* order, int32_t* states, void* locx0,
                               int64_t capacity, int64_t* count);

/* Medium coefficients per cell (alpha, beta, Q: [N] FP64 host arrays) and the
 * intensities of boundary codes -1..-4 (bc [4]; NULL: 0, 0, 1, 0 as
 * BoundaryConditions, solve_module/illum/illum_utils.cpp:407-474). */
int rts_sweep_set_medium(rts_ctx* ctx, const rts_medium* md, const double* alpha, const double* beta,
                         const double* Q, const double* bc);

/* Class 11 of GetCurIllum (Illum_async.cpp:419-447), the medium coupled to
 * the gas: for each cell, from its density and pressure in code units
 * (flux_t::d, flux_t::p), alpha = beta = d DENSITY sigma_thomson / m_hydrogen
 * and Q = alpha Ie(T), T = min(1e-6 p PRESSURE / (d DENSITY R_gas), 5000),
 * with the reference's units and constants (global_value.h:32-52); *md is set
 * to the scattering form with s_scale = DIST and i_scale = RADIATION.  Host
 * only.  Pass the result to rts_sweep_set_medium. */
int rts_sweep_medium_gas(int64_t N, const double* density, const double* pressure, double* alpha, double* beta,
                         double* Q, rts_medium* md);

/* One sweep of every local direction (the direction loops of
 * MPI_CalculateIllumAsync, solve_module/illum/Illum_async.cpp:726-784 and
 * 827-885) on `stream`: reads the device scattering array [local][N] and
 * writes the face means of the local directions' rows of the device Illum
 * (ReCalcIllum, :472-510).  *norm (may be NULL) receives ReCalcIllum's
 * max |old - new| / new over all faces (-1 if every term was NaN), which
 * synchronises the stream. */
int rts_sweep(rts_ctx* ctx, int stream, double* norm);

/* The source iteration of MPI_CalculateIllumAsync (Illum_async.cpp:615-1060)
 * on the device: repeat { sweep; if max_iter > 1, the scattering integral of
 * the new Illum into the device scattering array at `precision`
 * (rts_precision) } while norm > accuracy and fewer than max_iter sweeps ran.
 * norms [max_iter] (may be NULL) receives each sweep's norm, *iters the
 * sweeps run.  On RTS_STREAM_SCATTERING_1; one 8-byte read-back per sweep. */
int rts_illum_solve(rts_ctx* ctx, int precision, int max_iter, double accuracy, int64_t* iters, double* norms);

/* ---------------------------------------------------------------------- */
/* instrumentation                                                         */
/* ---------------------------------------------------------------------- */

/* Tuning knobs of the tensor-core path (0 restores the default):
 *   RTS_TUNE_FLUSH: K-slices (32 in-directions for FP16 / BF16, 16 for TF32)
 *   accumulated on the tensor core before the partial sum is added in FP32
 *   on the CUDA cores: 1 or 2.  The default (0) is automatic: for FP16 and
 *   BF16, 2 -- half as many drains -- only when no 16-direction block of any
 *   out-direction's column of W carries more than 1/8 of it (smooth kernels
 *   on enough directions: Thomson at M >= 302, Henyey-Greenstein with small
 *   g), else 1 (caller-supplied W: 1); for TF32 always 2 (32 in-directions
 *   per drain).
 *   RTS_TUNE_BIAS: correction of the tensor core's truncating FP32
 *   accumulation (each accumulate rounds toward zero, so sums come out low by
 *   ~1e-7 of themselves).  0 (default): relaxed source iterations scale each
 *   cell's integrals by (1 + delta), delta = sum_j v_j I_j / sum_k S_k - 1
 *   of that cell in the previous step (v = W 1 in FP64; the sum over k of
 *   the integrals is conserved), which removes the part of the loss that
 *   would compound; single evaluations keep the loss of one pass.  -1: no
 *   correction.  n > 0: the default plus a constant factor (1 + n * 1e-10)
 *   on every sum.  Takes effect for iterations set up (rts_solve_setup,
 *   rts_batch_add) after the change. */
#define RTS_TUNE_FLUSH 1
#define RTS_TUNE_BIAS 2
/*   RTS_TUNE_SERVE_POLICY: how rts_serve_run chooses the requests a step
 *   advances: 1 (default) earliest deadline first, the deadline being arrival
 *   + RTS_TUNE_SERVE_SLACK/100 x the request's estimated solve time alone; 2
 *   least remaining work first, a request left out gaining priority with
 *   every step it waits; 3 first come first served (the oldest request's
 *   whole step first, later ones only in the budget it leaves: a request
 *   whose step fills the budget runs alone); 1 to 3 within a tile budget; 0
 *   every resident request every step.
 *   RTS_TUNE_SERVE_BUDGET: tiles (128 cells x up to 256 directions) per step
 *   under policies 1 to 3; 0 = 8 waves of the SMs.  At least one request
 *   always runs. */
/*   RTS_TUNE_SERVE_SLACK: policy 1's deadline, arrival + slack/100 x the
 *   request's estimated solve time alone (0 = 500). */
#define RTS_TUNE_SERVE_POLICY 3
#define RTS_TUNE_SERVE_BUDGET 4
#define RTS_TUNE_SERVE_SLACK 5
/*   RTS_TUNE_SWEEP_CACHE: 1 (default) the first rts_sweep after a change of
 *   the medium or of the structures stores every node's attenuation factor
 *   exp(-k s) (8 bytes per node record, allocated then; within budget), and
 *   the sweeps after it read the factor instead of evaluating it -- the same
 *   numbers, without the exponential; 0 every sweep evaluates them (and the
 *   factors are not allocated).  A sweep that cannot allocate the factors
 *   evaluates them. */
#define RTS_TUNE_SWEEP_CACHE 6
int rts_set_tuning(rts_ctx* ctx, int key, int value);

/* The drain period (K-slices per FP32 drain) that the context's tensor-core
 * calls at `precision` use for its current directions, out-directions and
 * phase kernel: RTS_TUNE_FLUSH when set, else the automatic choice. */
int rts_flush_period(const rts_ctx* ctx, int precision, int* flush);

/* Autotuner of the tensor-core kernel's schedule: drain period (K-slices
 * per FP32 drain), tile width (out-directions per tile) and tile order.  No
 * counterpart in the reference (its launch shape is fixed).
 *
 * rts_autotune_schedule times, on a synthetic Thomson problem of `cells`
 * cells (0: four waves of 128-cell row tiles) and M Fibonacci directions at
 * `precision`, every drain period the accuracy rule allows (FP16 / BF16: 1,
 * and 2 where RTS_TUNE_FLUSH's automatic choice gives 2; TF32: 2), every
 * distinct tiling of the M out-directions (tiles of 64..256) and both tile
 * orders (0: the column tiles of a row tile in turn; 1: the row tiles of a
 * column tile in turn).  The fastest width and order of each period enter
 * the context's table under (M, precision, period, cell bucket), the bucket
 * being the cell count in waves of row tiles over the SMs (below 1, 4, 16,
 * or more).  Problems created afterwards -- batches, serving requests and the
 * context's own calls -- take, unless their caller fixes it (desc->flush,
 * RTS_TUNE_FLUSH), the allowed period with the shorter tuned time, and with
 * it, unless fixed (desc->bn), that period's width, and its order, from the
 * entry of the nearest bucket.  Width and order give bit-identical results;
 * the period changes the rounding within the accuracy the rule guarantees.
 * *best receives the fastest schedule; tried (capacity entries, may be NULL
 * when capacity is 0) every timing, *n_tried their count. */
typedef struct rts_tune_choice {
    int64_t M;
    int precision;
    int flush;   /* K-slices per drain */
    int bn;      /* out-directions per tile */
    int order;   /* 0: column tiles of a row tile in turn; 1: row tiles of a column tile */
    int bucket;  /* cell bucket of the timing problem */
    double ms;   /* one relaxed step of the timing problem */
} rts_tune_choice;
int rts_autotune_schedule(rts_ctx* ctx, int64_t M, int precision, int64_t cells, rts_tune_choice* best,
                          rts_tune_choice* tried, int capacity, int* n_tried);
/* The width-only search at one drain period (flush 0: the automatic one),
 * tile order 0; the fastest width enters the table as above.  tried_bn /
 * tried_ms (capacity entries, may be NULL) receive every timing, *tried their
 * count. */
int rts_autotune(rts_ctx* ctx, int64_t M, int precision, int flush, int64_t cells, int* best_bn, double* best_ms,
                 int* tried_bn, double* tried_ms, int capacity, int* tried);
/* The table as text ("M precision flush cell_bucket bn order ms" per line),
 * and back (tables of "M precision flush bn ms" lines load as entries for
 * every bucket, order 0). */
int rts_autotune_save(rts_ctx* ctx, const char* path);
int rts_autotune_load(rts_ctx* ctx, const char* path);

/* The cudaStream_t of a stream slot (for callers that order their own work
 * or record CUDA events against the library's streams). */
int rts_stream_handle(rts_ctx* ctx, int stream, void** handle);

/* Self-check of the sweep's FP64 exponential (a table-driven method for
 * arguments in [-700, 0]) against CUDA's exp at n points of that range:
 * *max_ulp receives the largest difference in units in the last place. */
int rts_sweep_exp_check(rts_ctx* ctx, int64_t n, double* max_ulp);

/* Measured ceilings for roofline fractions (no counterpart in the
 * reference).  rts_measure_fp64_peak: FP64 FMA throughput of the device in
 * TFLOP/s (2 flops per FMA), from independent FMA chains on every SM timed
 * with CUDA events over about `seconds`.  rts_measure_link: pinned host <->
 * device copy rates in GB/s for copies of `bytes`, best of `reps`: H2D alone,
 * D2H alone, and both directions at once (bytes moved both ways / time).
 * Each allocates its buffers for the duration of the call. */
int rts_measure_fp64_peak(rts_ctx* ctx, double seconds, double* tflops);
int rts_measure_link(rts_ctx* ctx, int64_t bytes, int reps, double* h2d_gbs, double* d2h_gbs, double* both_gbs);

/* Number of kernels this context has launched so far. */
int rts_launch_count(const rts_ctx* ctx, int64_t* count);

/* CUDA-event timing of the dominant kernel of each integral (the FP64
 * scattering kernel or the tensor-core contraction), recorded on the stream
 * it is launched on.  enable != 0 turns recording on and clears the totals;
 * total_ms / launches (may be NULL) return what was recorded so far, after
 * synchronising the recorded events. */
int rts_kernel_timing(rts_ctx* ctx, int enable, double* total_ms, int64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* RTS_SCATTER_H */
