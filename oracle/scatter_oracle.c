/*
 * scatter_oracle.c -- CPU oracle for the scattering-integral path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file.  It is used by tests/ (as the checker), by
 * __graft_entry__.smoke() (as the checker) and by bench.py's CPU-baseline leg
 * (as the timed reference CPU implementation).
 *
 * What it restates (reference paths are relative to solver_hllc_illum_cuda/):
 *   orc_gets ............ GetS             solve_module/illum/Illum_async.cpp:201-232
 *   orc_calculate_int_cpu CalculateIntCPU  solve_module/illum/Illum_async.cpp:234-256
 *   orc_energy .......... GET_FACE_TO_CELL + IntegarteDirection
 *                                         solve_module/illum/Illum_async.cpp:1101-1122
 *   orc_stream .......... IntegarteDirection3 + GET_FACE_TO_CELL (MakeStream)
 *                                         solve_module/illum/Illum_async.cpp:1156-1178,1197
 *   orc_get_send/_disp .. GetSend / GetDisp solve_module/solve_utils.cpp:177-202
 *   Gamma (inline) ...... lambda in GetS   solve_module/illum/Illum_async.cpp:203-206
 *                         device twin      cuda/cuda_utils.cu:7-16
 * Loop order and operation order follow the reference: out-direction k
 * (OpenMP), then cell, then in-direction j; the face mean adds faces 0..3 in
 * order to a zero start and divides by 4; S += (Gamma * I) * area_j; the
 * division by full_area comes last.  Deviations: 64-bit indices (the
 * reference's int indices overflow at 4*N*M > 2^31) and a plain x,y,z dot
 * product in place of Eigen's Vector3d::dot.
 *
 * Parity pin: the reference's own GetS / CalculateIntCPU source, compiled in
 * the development container by oracle/build_ref.sh against a small stand-in
 * for the Eigen / MPI / grid types, produced the golden vectors in
 * tests/golden/; tests/test_oracle.py checks this restatement against them.
 *
 * The synthetic-input helpers (Fibonacci directions, counter-based lognormal
 * intensities, Thomson / Henyey-Greenstein weight matrices) define the
 * workloads the tests and the benchmark share; the CUDA library has its own
 * device-side generator that uses the same counter hash.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_BASE 4 /* faces per tetrahedron: `base` in global_def.h:23 */

/* ------------------------------------------------------------------ */
/* counter-based random numbers (splitmix64 finaliser)                 */
/* ------------------------------------------------------------------ */
static inline uint64_t orc_mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* uniform in (0,1): 53 random bits, centred so 0 and 1 never occur */
double orc_uniform(uint64_t seed, uint64_t stream, uint64_t idx)
{
    uint64_t key = orc_mix64(seed * 0x632BE59BD9B4E019ull + stream);
    uint64_t r = orc_mix64(key ^ orc_mix64(idx));
    return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

/* standard normal by Box-Muller on the index pair (2*idx, 2*idx+1) */
double orc_normal(uint64_t seed, uint64_t stream, uint64_t idx)
{
    const double two_pi = 6.283185307179586476925286766559;
    double u1 = orc_uniform(seed, stream, 2 * idx);
    double u2 = orc_uniform(seed, stream, 2 * idx + 1);
    return sqrt(-2.0 * log(u1)) * cos(two_pi * u2);
}

/* Illum[j][c][f] for j in [j0, j1) of an N-cell, M-direction problem.
 * One lognormal draw per (cell, direction) replicated into the 4 face slots,
 * or (independent_faces != 0) one draw per face.  Output holds
 * (j1 - j0) * N * 4 doubles, direction-major as in grid_t::Illum. */
void orc_fill_illum(uint64_t seed, double mu, double sigma, int64_t N,
                    int64_t j0, int64_t j1, int independent_faces, double* out)
{
    const int64_t rows = j1 - j0;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < rows; ++r) {
        const int64_t j = j0 + r;
        for (int64_t c = 0; c < N; ++c) {
            double* dst = out + (r * N + c) * ORC_BASE;
            if (independent_faces) {
                for (int f = 0; f < ORC_BASE; ++f)
                    dst[f] = exp(mu + sigma * orc_normal(seed, 1, ((uint64_t)(j * N + c)) * ORC_BASE + f));
            } else {
                double v = exp(mu + sigma * orc_normal(seed, 1, (uint64_t)(j * N + c)));
                for (int f = 0; f < ORC_BASE; ++f) dst[f] = v;
            }
        }
    }
}

/* Same values as orc_fill_illum, written only for cells [c0, c1) of the
 * full [M][N][4] array `out` (other entries untouched): lets a bounded CPU
 * sample run the integral with the full problem's strides. */
void orc_fill_illum_cells(uint64_t seed, double mu, double sigma, int64_t N, int64_t M,
                          int64_t c0, int64_t c1, int independent_faces, double* out)
{
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < M; ++j)
        for (int64_t c = c0; c < c1; ++c) {
            double* dst = out + (j * N + c) * ORC_BASE;
            if (independent_faces) {
                for (int f = 0; f < ORC_BASE; ++f)
                    dst[f] = exp(mu + sigma * orc_normal(seed, 1, ((uint64_t)(j * N + c)) * ORC_BASE + f));
            } else {
                double v = exp(mu + sigma * orc_normal(seed, 1, (uint64_t)(j * N + c)));
                for (int f = 0; f < ORC_BASE; ++f) dst[f] = v;
            }
        }
}

/* uniform(lo, hi) values on stream `stream`, indices [i0, i0 + n) */
void orc_fill_normal(uint64_t seed, uint64_t stream, int64_t n, double* out)
{
    for (int64_t i = 0; i < n; ++i) out[i] = orc_normal(seed, stream, (uint64_t)i);
}

void orc_fill_uniform(uint64_t seed, uint64_t stream, double lo, double hi,
                      int64_t i0, int64_t n, double* out)
{
    for (int64_t i = 0; i < n; ++i)
        out[i] = lo + (hi - lo) * orc_uniform(seed, stream, (uint64_t)(i0 + i));
}

/* ------------------------------------------------------------------ */
/* direction sets and direction-pair weights                           */
/* ------------------------------------------------------------------ */

/* spherical Fibonacci points: z_i = 1-(2i+1)/M, phi_i = i*pi*(3-sqrt 5);
 * weights 4*pi/M, full_area 4*pi (the direction-file layout of
 * file_module/reader_txt.cpp:25-47: area, x, y, z per line). */
void orc_fibonacci_directions(int64_t M, double* xyz, double* area, double* full_area)
{
    const double pi = 3.14159265358979323846264338327950288;
    const double golden = pi * (3.0 - sqrt(5.0));
    for (int64_t i = 0; i < M; ++i) {
        double z = 1.0 - (2.0 * (double)i + 1.0) / (double)M;
        double r = sqrt(fmax(0.0, 1.0 - z * z));
        double phi = golden * (double)i;
        xyz[3 * i + 0] = r * cos(phi);
        xyz[3 * i + 1] = r * sin(phi);
        xyz[3 * i + 2] = z;
        area[i] = 4.0 * pi / (double)M;
    }
    *full_area = 4.0 * pi;
}

static inline double orc_gamma(const double* a, const double* b)
{
    /* cuda/cuda_utils.cu:7-16: dot in x, y, z order, then 3*(1+d*d)/4 */
    double dot = 0.0;
    dot += a[0] * b[0];
    dot += a[1] * b[1];
    dot += a[2] * b[2];
    return (3. * (1 + dot * dot)) / 4;
}

/* Thomson weights in the reference's form:
 * W[j][k] = Gamma(w_j, w_k) * area_j / full_area, j in-direction (row),
 * k out-direction (column), out-directions [k0, k0 + Mout). */
void orc_weights_thomson(int64_t M, const double* xyz, const double* area, double full_area,
                         int64_t k0, int64_t Mout, double* W)
{
    for (int64_t j = 0; j < M; ++j)
        for (int64_t k = 0; k < Mout; ++k)
            W[j * Mout + k] = orc_gamma(xyz + 3 * j, xyz + 3 * (k0 + k)) * area[j] / full_area;
}

/* Henyey-Greenstein weights renormalised per out-direction:
 * W[j][k] = w_j K(w_j.w_k) / sum_j' w_j' K(w_j'.w_k),
 * K(mu) = (1-g^2) / (4 pi (1+g^2-2 g mu)^{3/2}), so every column sums to 1. */
void orc_weights_hg(int64_t M, const double* xyz, const double* area, double g,
                    int64_t k0, int64_t Mout, double* W)
{
    const double pi = 3.14159265358979323846264338327950288;
    for (int64_t k = 0; k < Mout; ++k) {
        const double* b = xyz + 3 * (k0 + k);
        double colsum = 0.0;
        for (int64_t j = 0; j < M; ++j) {
            const double* a = xyz + 3 * j;
            double mu = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
            double den = 1.0 + g * g - 2.0 * g * mu;
            double kv = (1.0 - g * g) / (4.0 * pi * den * sqrt(den));
            double w = area[j] * kv;
            W[j * Mout + k] = w;
            colsum += w;
        }
        for (int64_t j = 0; j < M; ++j) W[j * Mout + k] /= colsum;
    }
}

/* ------------------------------------------------------------------ */
/* the scattering integral                                             */
/* ------------------------------------------------------------------ */

/* GetS (Illum_async.cpp:201-232).  num_cell is base*cell as in the caller;
 * Illum is [M][N][4]. */
double orc_gets(const double* illum, int64_t N, int64_t M, const double* xyz,
                const double* area, double full_area, const double* direction,
                int64_t num_cell)
{
    double S = 0;
    const int64_t N_cell = N * ORC_BASE;
    for (int64_t num_direction = 0; num_direction < M; num_direction++) {
        double I = 0;
        for (int i = 0; i < ORC_BASE; i++)
            I += illum[num_direction * N_cell + num_cell + i];
        I /= ORC_BASE;
        S += orc_gamma(xyz + 3 * num_direction, direction) * I * area[num_direction];
    }
    return S / full_area;
}

/* CalculateIntCPU (Illum_async.cpp:234-256): out-directions
 * [disp_loc, disp_loc + size_loc), written to scattering[k_local*N + cell]. */
void orc_calculate_int_cpu(int64_t N, int64_t M, const double* xyz, const double* area,
                           double full_area, const double* illum, int64_t disp_loc,
                           int64_t size_loc, double* scattering, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t k = 0; k < size_loc; ++k) {
        const double* direction = xyz + 3 * (disp_loc + k);
        for (int64_t cell = 0; cell < N; cell++)
            scattering[k * N + cell] =
                orc_gets(illum, N, M, xyz, area, full_area, direction, ORC_BASE * cell);
    }
    (void)nthreads;
}

/* Same integral for a subset of cells (used to sample large problems). */
void orc_calculate_int_cells(int64_t N, int64_t M, const double* xyz, const double* area,
                             double full_area, const double* illum, int64_t disp_loc,
                             int64_t size_loc, const int64_t* cells, int64_t ncells,
                             double* out /* [size_loc][ncells] */, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t k = 0; k < size_loc; ++k) {
        const double* direction = xyz + 3 * (disp_loc + k);
        for (int64_t i = 0; i < ncells; i++)
            out[k * ncells + i] =
                orc_gets(illum, N, M, xyz, area, full_area, direction, ORC_BASE * cells[i]);
    }
    (void)nthreads;
}

/* matrix form: out[k][c] = sum_j W[j][k] * Ibar[j][c]; FP64, j ascending */
void orc_scatter_matrix(const double* W, int64_t Min, int64_t Mout, const double* Ibar,
                        int64_t N, double* out, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t k = 0; k < Mout; ++k) {
        double* row = out + k * N;
        for (int64_t c = 0; c < N; ++c) row[c] = 0.0;
        for (int64_t j = 0; j < Min; ++j) {
            const double w = W[j * Mout + k];
            const double* src = Ibar + j * N;
            for (int64_t c = 0; c < N; ++c) row[c] += w * src[c];
        }
    }
    (void)nthreads;
}

/* face mean Ibar[j][c] = ((I0+I1)+I2+I3)/4 as GET_FACE_TO_CELL does */
void orc_face_mean(const double* illum, int64_t N, int64_t M, double* Ibar)
{
    for (int64_t j = 0; j < M; ++j)
        for (int64_t c = 0; c < N; ++c) {
            const double* s = illum + (j * N + c) * ORC_BASE;
            double I = 0;
            for (int f = 0; f < ORC_BASE; ++f) I += s[f];
            Ibar[j * N + c] = I / ORC_BASE;
        }
}

/* ------------------------------------------------------------------ */
/* direction moments                                                   */
/* ------------------------------------------------------------------ */

/* energy (Illum_async.cpp:1101-1122): E[c] = sum_j Ibar*area_j / full_area */
void orc_energy(const double* illum, int64_t N, int64_t M, const double* area,
                double full_area, double* energy)
{
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < N; ++c) {
        double res = 0;
        for (int64_t j = 0; j < M; ++j) {
            const double* s = illum + (j * N + c) * ORC_BASE;
            double I = 0;
            for (int f = 0; f < ORC_BASE; ++f) I += s[f];
            I /= ORC_BASE;
            res += I * area[j];
        }
        energy[c] = res / full_area;
    }
}

/* flux (Illum_async.cpp:1156-1178, face mean as MakeStream :1197): per-face
 * stream_f = sum_j I_f * area_j * w_j / full_area, then the face mean. */
void orc_stream(const double* illum, int64_t N, int64_t M, const double* xyz,
                const double* area, double full_area, double* stream /* N x 3 */)
{
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < N; ++c) {
        double sf[ORC_BASE][3];
        memset(sf, 0, sizeof(sf));
        for (int64_t j = 0; j < M; ++j) {
            const double* s = illum + (j * N + c) * ORC_BASE;
            for (int f = 0; f < ORC_BASE; ++f) {
                double ia = s[f] * area[j];
                sf[f][0] += ia * xyz[3 * j + 0];
                sf[f][1] += ia * xyz[3 * j + 1];
                sf[f][2] += ia * xyz[3 * j + 2];
            }
        }
        for (int d = 0; d < 3; ++d) {
            double v = 0;
            for (int f = 0; f < ORC_BASE; ++f) v += sf[f][d] / full_area;
            stream[3 * c + d] = v / ORC_BASE;
        }
    }
}

/* Flux, impulse tensor and their divergences (the reference's
 * d_MakeIllumParam: cuda/cuda_kernel.cu:149-175 d_MakeDivStream, :177-216
 * d_MakeDivImpuls, with IntegarteDirection3Faces / IntegarteDirection9Faces
 * of cuda/cuda_utils.cu:86-167 and the face mean CUDA_CONVERT_FATE_TO_CELL
 * of cuda/cuda_kernel.cu:9-17; CPU twins MakeStream / MakeDivImpuls at
 * solve_module/illum/Illum_async.cpp:1179-1349).  Per cell c and face f:
 *   Stream_f   = sum_j (I[j][c][f] * area_j) * w_j / full_area
 *   Impuls_f   = sum_j w_j w_j^T * (I[j][c][f] * area_j) / full_area
 * flux and impuls are the face means; with the cell's outward face normals
 * n_f, face areas S_f and volume V:
 *   divstream  = sum_f (Stream_f . n_f) S_f / V
 *   divimpuls  = sum_f (Impuls_f n_f) S_f / V
 * Outputs: flux [N][3], impuls [N][9] (row-major h*3+k), divstream [N],
 * divimpuls [N][3]; any may be NULL. */
void orc_illum_params(const double* illum, int64_t N, int64_t M, const double* xyz, const double* area,
                      double full_area, const double* normals /* N x 4 x 3 */,
                      const double* face_areas /* N x 4 */, const double* volume, double* flux,
                      double* impuls, double* divstream, double* divimpuls)
{
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < N; ++c) {
        double st[ORC_BASE][3], im[ORC_BASE][9];
        memset(st, 0, sizeof(st));
        memset(im, 0, sizeof(im));
        for (int64_t j = 0; j < M; ++j) {
            const double* s = illum + (j * N + c) * ORC_BASE;
            const double* w = xyz + 3 * j;
            for (int f = 0; f < ORC_BASE; ++f) {
                const double ia = s[f] * area[j];
                for (int d = 0; d < 3; ++d) st[f][d] += w[d] * ia;
                for (int h = 0; h < 3; ++h)
                    for (int k = 0; k < 3; ++k) im[f][h * 3 + k] += w[h] * w[k] * ia;
            }
        }
        for (int f = 0; f < ORC_BASE; ++f) {
            for (int d = 0; d < 3; ++d) st[f][d] /= full_area;
            for (int d = 0; d < 9; ++d) im[f][d] /= full_area;
        }
        if (flux)
            for (int d = 0; d < 3; ++d) {
                double v = 0;
                for (int f = 0; f < ORC_BASE; ++f) v += st[f][d];
                flux[3 * c + d] = v / ORC_BASE;
            }
        if (impuls)
            for (int d = 0; d < 9; ++d) {
                double v = 0;
                for (int f = 0; f < ORC_BASE; ++f) v += im[f][d];
                impuls[9 * c + d] = v / ORC_BASE;
            }
        const double* n = normals + 12 * c;
        const double* S = face_areas + 4 * c;
        if (divstream) {
            double v = 0;
            for (int f = 0; f < ORC_BASE; ++f) {
                double dot = 0;
                for (int k = 0; k < 3; ++k) dot += st[f][k] * n[3 * f + k];
                v += dot * S[f];
            }
            divstream[c] = v / volume[c];
        }
        if (divimpuls)
            for (int h = 0; h < 3; ++h) {
                double v = 0;
                for (int f = 0; f < ORC_BASE; ++f) {
                    double dot = 0;
                    for (int k = 0; k < 3; ++k) dot += im[f][h * 3 + k] * n[3 * f + k];
                    v += dot * S[f];
                }
                divimpuls[3 * c + h] = v / volume[c];
            }
    }
}

/* ------------------------------------------------------------------ */
/* source update, relaxation and residual                              */
/* ------------------------------------------------------------------ */

/* S <- (1-lambda) B + lambda S, B per cell, S [k][c] */
void orc_source_update(int64_t N, int64_t Mout, double* S, const double* B, double lambda)
{
    for (int64_t k = 0; k < Mout; ++k)
        for (int64_t c = 0; c < N; ++c)
            S[k * N + c] = (1.0 - lambda) * B[c] + lambda * S[k * N + c];
}

double orc_max_abs_diff(const double* a, const double* b, int64_t n)
{
    double m = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double d = fabs(a[i] - b[i]);
        if (d > m) m = d;
    }
    return m;
}

/* Per-cell source iteration in FP64 on Ibar rows (cells are independent):
 *   S_int = W^T Ibar;  S = (1-lambda) B + lambda S_int;
 *   residual_it = max |S - S_prev|   (S_prev = 0 before the first step);
 *   Ibar <- 0.5 Ibar + 0.5 S   (only when M_in == M_out).
 * Ibar [M][ncell] is updated in place; S [M][ncell] holds the last S;
 * residual[it] per iteration. */
void orc_iterate(const double* W, int64_t M, double* Ibar, int64_t ncell, const double* B,
                 double lambda, int iters, int relax, double* S, double* residual)
{
    double* tmp = (double*)malloc(sizeof(double) * (size_t)(M * ncell));
    for (int64_t i = 0; i < M * ncell; ++i) S[i] = 0.0;
    for (int it = 0; it < iters; ++it) {
        orc_scatter_matrix(W, M, M, Ibar, ncell, tmp, 1);
        double res = 0.0;
        for (int64_t k = 0; k < M; ++k)
            for (int64_t c = 0; c < ncell; ++c) {
                double v = (1.0 - lambda) * B[c] + lambda * tmp[k * ncell + c];
                double d = fabs(v - S[k * ncell + c]);
                if (d > res) res = d;
                S[k * ncell + c] = v;
            }
        residual[it] = res;
        if (relax)
            for (int64_t i = 0; i < M * ncell; ++i) Ibar[i] = 0.5 * Ibar[i] + 0.5 * S[i];
    }
    free(tmp);
}

/* ------------------------------------------------------------------ */
/* direction partition (solve_module/solve_utils.cpp:177-202)          */
/* ------------------------------------------------------------------ */
void orc_get_send(int np, int n, int* send_count)
{
    for (int i = 0; i < np; ++i) send_count[i] = n / np;
    if (n % np)
        for (int i = 0; i < n % np; i++) ++send_count[i];
}

void orc_get_disp(int np, int n, int* disp)
{
    int a = n % np;
    disp[0] = 0;
    for (int i = 1; i < np; i++) disp[i] = i * (n / np) + a;
    if (n % np)
        for (int i = 1; i < a; i++) disp[a - i] -= i;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
