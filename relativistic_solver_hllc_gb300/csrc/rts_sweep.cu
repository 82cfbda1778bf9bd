// rts_sweep.cu -- the transport sweep that produces Illum, on the device.
//
// For every direction the reference walks the cells in dependency order
// (Illum_async.cpp:726-784): at each out-face node it takes the mean of the
// in-face the characteristic comes from, integrates GetCurIllum over the
// distance s to it, and stores the three node values of the face for the
// face and its neighbour's copy; ReCalcIllum then writes the face means into
// Illum and measures the change.  Here:
//   - the dependency order is cut into steps (build_graph's steps: cells
//     whose in-faces are all known), computed on the host, and one CTA per
//     direction walks the steps with a barrier between them;
//   - the unit of work within a step is an out-face (always 3 nodes, so the
//     lanes of a warp stay busy; a thread per cell would idle half its lanes
//     on the faces that are in-faces of its cell), and its 3 node distances
//     are the LocX0 records in the order the reference writes them;
//   - the in-face value a node needs is exactly the face mean its upstream
//     cell wrote, so only face means are kept, straight in the device Illum
//     [dir][cell][face] (the reference's node triples are never stored), and
//     ReCalcIllum's norm is taken as each face is written;
//   - the geometry (in-face and distance of every node) is built once per
//     mesh and direction set by a device kernel.
// Reference paths are relative to solver_hllc_illum_cuda/.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "rts_internal.h"

void rts_face_normals_host(int64_t N, const double* vert, double* normals);
void rts_sweep_nodes_host(int64_t N, const double* vert, double* nodes);

namespace {

// 128 threads and at most 72 registers: 7 CTAs per SM, so one wave of 152 x 7
// CTAs holds 1000 directions (the sweep is bound by the FP64 pipe; a second
// partial wave cost 11 %).
constexpr int SWEEP_THREADS = 128;
constexpr double SWEEP_EPS = 1e-10;  // `eps`, global_value.h:13
constexpr int kExpTable = 256;       // entries 2^(j/256) of the sweep's exponential (exp_neg)

__host__ __device__ inline void face_verts(int f, int& a, int& b, int& c)
{
    // VTK's tetra faces {0,1,3}, {1,2,3}, {2,0,3}, {0,2,1}
    a = f == 1 ? 1 : f == 2 ? 2 : 0;
    b = f == 0 ? 1 : f == 1 ? 2 : f == 2 ? 0 : 2;
    c = f == 3 ? 1 : 3;
}

// ---------------------------------------------------------------- geometry

// Everything about an in-face that the characteristic test needs and that
// does not depend on the direction or the node, computed once per face:
//   [0..3]   the plane a x + b y + c z + d = 0 through A, B, C with the
//            coefficients IntersectionWithPlane forms
//            (utils/grid_geometry/geometry_solve.cpp:109-128);
//   [4..9]   the plane frame v1, v2 of SetBasis (:8-43) for the cell's
//            outward face normal n;
//   [10..13] B and C in that frame (Make2dPoint, :45-56, relative to A; A
//            itself maps to (0, 0)).
constexpr int kFrame = 16;  // doubles per face (14 used)

__device__ inline void face_frame(const double* A, const double* B, const double* C, const double* n, double* F)
{
    F[0] = A[1] * (B[2] - C[2]) + B[1] * (C[2] - A[2]) + C[1] * (A[2] - B[2]);
    F[1] = A[0] * (C[2] - B[2]) + B[0] * (A[2] - C[2]) + C[0] * (B[2] - A[2]);
    F[2] = A[0] * (B[1] - C[1]) + B[0] * (C[1] - A[1]) + C[0] * (A[1] - B[1]);
    F[3] = A[0] * (C[1] * B[2] - B[1] * C[2]) + B[0] * (A[1] * C[2] - C[1] * A[2]) +
           C[0] * (B[1] * A[2] - A[1] * B[2]);
    double v1[3], v2[3];
    if (fabs(n[1]) < 1e-20) {
        v1[0] = 0, v1[1] = 1, v1[2] = 0;
    } else {
        v1[0] = 1, v1[2] = 0;
        v1[1] = -(n[0] * v1[0] + n[2] * v1[2]) / n[1];
    }
    if (n[1] < 0)
        for (int i = 0; i < 3; ++i) v1[i] = -v1[i];
    v2[0] = -(n[1] * v1[2] - n[2] * v1[1]);
    v2[1] = -(n[2] * v1[0] - n[0] * v1[2]);
    v2[2] = -(n[0] * v1[1] - n[1] * v1[0]);
    const double z1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    const double z2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
    for (int i = 0; i < 3; ++i) v1[i] /= z1, v2[i] /= z2;
    const double* P[2] = {B, C};
    for (int p = 0; p < 2; ++p) {
        double u = 0, w = 0;
        for (int k = 0; k < 3; ++k) {
            u += (P[p][k] - A[k]) * v1[k];
            w += (P[p][k] - A[k]) * v2[k];
        }
        F[10 + 2 * p] = u, F[11 + 2 * p] = w;
    }
    for (int i = 0; i < 3; ++i) F[4 + i] = v1[i], F[7 + i] = v2[i];
}

__global__ void __launch_bounds__(256) sweep_frames_kernel(const double* __restrict__ vert,
                                                           const double* __restrict__ normals, int64_t N,
                                                           double* __restrict__ frames)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 4 * N; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = i >> 2;
        const int g = (int)(i & 3);
        int ia, ib, ic;
        face_verts(g, ia, ib, ic);
        const double* v = vert + 12 * c;
        face_frame(v + 3 * ia, v + 3 * ib, v + 3 * ic, normals + 3 * i, frames + kFrame * i);
    }
}

// The characteristic from node x back along dir meets the plane of in-face F
// at X (IntersectionWithPlane); InTriangle (geometry_solve.cpp:129-159):
// X strictly inside the triangle, in the face's 2-D frame.
__device__ inline bool hits_face(const double* __restrict__ F, const double* A, const double* x, const double* dir,
                                 double* X)
{
    const double t = -(F[0] * x[0] + F[1] * x[1] + F[2] * x[2] + F[3]) / (F[0] * dir[0] + F[1] * dir[1] + F[2] * dir[2]);
    for (int i = 0; i < 3; ++i) X[i] = dir[i] * t + x[i];
    double u = 0, w = 0;
    for (int k = 0; k < 3; ++k) {
        u += (X[k] - A[k]) * F[4 + k];
        w += (X[k] - A[k]) * F[7 + k];
    }
    const double bu = F[10], bw = F[11], cu = F[12], cw = F[13];
    const double r1 = (0.0 - u) * (bw - 0.0) - (bu - 0.0) * (0.0 - w);
    const double r2 = (bu - u) * (cw - bw) - (cu - bu) * (bw - w);
    const double r3 = (cu - u) * (0.0 - cw) - (0.0 - cu) * (cw - w);
    return (r1 < 0 && r2 < 0 && r3 < 0) || (r1 > 0 && r2 > 0 && r3 > 0);
}

struct X0Args {
    const double* vert;      // [N][4][3]
    const double* frames;    // [N][4][kFrame]
    const double* nodes;     // [N][4][3][3]
    const double* dirs;      // [D][3]
    const uint8_t* states;   // [D][N] in-face flags
    uint32_t* const* items;  // [D]
    double* const* recs;     // [D]
    double* const* att;      // [D] attenuation factors, parallel to recs (stored or read by the cached forms)
    int32_t* const* steps;   // [D]
    const int32_t* nsteps;   // [D]
    int64_t N;
    int64_t d0;              // first direction of this launch (grid y covers at most 65535)
    int* flag;               // set when a node finds no in-face
};

// CalculateNodeValue (make_illum_struct/struct_short_characteristics_logic_function.cpp:
// 222-254) for the 3 nodes of every item: the first in-face, in face order,
// whose triangle contains the back-traced point, and the distance to it.
// Grid: x over the items of a direction, y over the directions.
__global__ void __launch_bounds__(256) sweep_x0_kernel(X0Args a)
{
    const int64_t d = a.d0 + blockIdx.y;
    const int64_t n = a.steps[d][a.nsteps[d]];
    uint32_t* items = a.items[d];
    double* recs = a.recs[d];
    const double* dir = a.dirs + 3 * d;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t w = items[i];
        const int64_t c = w >> 8;
        const int f = (int)((w >> 6) & 3u);
        const int st = a.states[d * a.N + c];
        const double* v = a.vert + 12 * c;
        for (int m = 0; m < 3; ++m) {
            const double* x = a.nodes + 36 * c + 9 * f + 3 * m;
            int found = -1, first_in = -1;
            double sv = 0.0;
            for (int g = 0; g < 4 && found < 0; ++g) {
                if (!((st >> g) & 1)) continue;
                if (first_in < 0) first_in = g;
                int ia, ib, ic;
                face_verts(g, ia, ib, ic);
                double x0[3];
                if (hits_face(a.frames + kFrame * (4 * c + g), v + 3 * ia, x, dir, x0)) {
                    const double d0 = x[0] - x0[0], d1 = x[1] - x0[1], d2 = x[2] - x0[2];
                    sv = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                    found = g;
                }
            }
            if (found < 0) {
                atomicOr(a.flag, 1);
                found = first_in < 0 ? 0 : first_in;
            }
            recs[3 * i + m] = sv;
            w |= (uint32_t)found << (2 * m);
        }
        items[i] = w;
    }
}

// ---------------------------------------------------------------- sweep

struct SweepArgs {
    uint32_t* const* items;  // [D]
    double* const* recs;     // [D]
    double* const* att;      // [D] attenuation factors, parallel to recs (stored or read by the cached forms)
    int32_t* const* steps;   // [D]
    uint32_t* const* bnd;    // [D]
    const int32_t* nsteps;   // [D]
    const int32_t* nbnd;     // [D]
    const int32_t* pairs;    // [N][4]
    const double* nodes;     // [N][4][3][3] (read only with a ball)
    const double* med;       // [N][4] k, beta, Q, 1/k
    const double* S;         // [D][N]
    double* illum;           // [D][N][4], rows of the local directions
    int64_t N;
    rts_medium md;
    double bc[4];
    double exp2tab[kExpTable];  // 2^(j/256)
    double ball[4];          // medium table entry of the ball's coefficients
    unsigned long long* norm;
};

// exp(x) for -700 <= x <= 0 by Tang's table-driven method (P. T. P. Tang,
// "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15(2), 1989): x = (256 m + j) ln2/256
// + r with |r| <= ln2/512, exp(x) = 2^m 2^(j/256) (1 + p(r)), 2^(j/256) from
// a 256-entry table and 2^m added to the exponent field.  p(r) = r + r^2 h(r)
// with h the quadratic fitted to (exp(r) - 1 - r) / r^2 on that interval by
// weighted least squares at Chebyshev nodes (relative error of 1 + p below
// 5.1e-18, against 1.1e-16 for one ulp).  9 FP64 operations against the
// general exp's range checks and longer polynomial; within 1.03 ulp of the
// exact value over the range (checked against CUDA's exp by
// rts_sweep_exp_check).
constexpr double kExpInvL = 369.3299304675746;            // 256 / ln 2
constexpr double kExpLHi = 0.0027076061740622863;         // ln 2 / 256, leading part
constexpr double kExpLLo = 9.058776616587108e-20;         // ln 2 / 256 - kExpLHi
constexpr double kExpShift = 6755399441055744.0;          // 1.5 * 2^52: rounds to an integer
constexpr double kExpH0 = 0.49999999999999795, kExpH1 = 0.16666668003070842, kExpH2 = 0.04166667023041113;

__device__ __forceinline__ double exp_neg(double x, const double* __restrict__ tab)
{
    const double t = fma(x, kExpInvL, kExpShift);
    const int n = __double2loint(t);
    const double N = t - kExpShift;
    double r = fma(-N, kExpLHi, x);
    r = fma(-N, kExpLLo, r);
    const double h = fma(r, fma(r, kExpH2, kExpH1), kExpH0);
    const double p = fma(r * r, h, r);
    const double T = tab[n & (kExpTable - 1)];
    const double y = fma(T, p, T);
    return __longlong_as_double(__double_as_longlong(y) + ((long long)(n >> 8) << 52));
}

// Per-cell terms of GetCurIllum (solve_module/illum/Illum_async.cpp:259-470):
// scattering form k = alpha + beta, R = Q + S' beta; absorption form
// k = alpha, R = Q; ks = k * s_scale, Rk = R / k.  The medium table keeps k,
// beta (0 in the absorption form), Q and 1 / k per cell, so that neither an
// item nor a node adds or divides for them.
struct CellTerms {
    double k, ks, R, Rk;
};

__device__ inline CellTerms cell_terms(const rts_medium& md, bool unit_i, bool unit_s, double k, double betta,
                                       double Q, double inv_k, double S)
{
    CellTerms t;
    t.k = k;
    t.R = Q + (unit_i ? S : S * md.i_scale) * betta;
    t.ks = unit_s ? k : k * md.s_scale;
    t.Rk = t.R * inv_k;
    return t;
}

// the table entry (k, beta, Q, 1/k) of coefficients alpha, beta, Q
__host__ __device__ inline void medium_entry(int mode, double alpha, double betta, double Q, double* e)
{
    const double k = mode == RTS_MEDIUM_ABSORPTION ? alpha : alpha + betta;
    e[0] = k;
    e[1] = mode == RTS_MEDIUM_ABSORPTION ? 0.0 : betta;
    e[2] = Q;
    e[3] = k != 0.0 ? 1.0 / k : 0.0;  // k = 0: those nodes take the reference's expression
}

// The reference's own expressions, for the nodes outside the fast path
// (kept out of line: they are rare and their exponentials cost registers).
__device__ __noinline__ double node_illum_ref(int mode, double k, double ss, double I0, double R)
{
    if (mode == RTS_MEDIUM_ABSORPTION) {
        if (k > 1e-15) return I0 * exp(-k * ss) + R * (1 - exp(-k * ss)) / k;
        return I0 * (1 - k * ss) + R * ss;
    }
    if (k > 1e-10) return (exp(-k * ss) * (I0 * k + (exp(k * ss) - 1) * R)) / k;
    return (1 - ss * k) * (I0 + ss * R);
}

// The fast range 1e-3 <= x <= 700 as bounds on the high word of x (x >= 0,
// and non-negative doubles order as their bit patterns): integer compares,
// off the FP64 pipe.  The bounds are 1e-3 - 8e-10 and 700 + 1e-13.
constexpr int kFastXLo = 0x3F50624D;  // high word of 1e-3
constexpr int kFastXHi = 0x4085E000;  // high word of 700

// GetCurIllum for one node at distance s from the in-face value I_0.  The
// reference evaluates exp(-x) (I0 k + (exp(x) - 1) R) / k, x = k s (the
// scattering form) or I0 exp(-x) + R (1 - exp(-x)) / k (the absorption
// form); where 1e-3 <= x <= 700 both are evaluated as e I0 + (1 - e) R / k
// with e = exp(-x) -- the same number up to a few ulp (the reference and this
// form both lose ~eps / x to the cancellation in exp(x) - 1, resp. 1 - e) for
// one exponential and no division per node, the dominant FP64 cost.  Outside
// that range the reference's own expression runs (including its overflow
// past x = 709).
//
// The node's attenuation factor e depends on the medium and the node's
// distance only, not on I_0 or the source S: node_att gives e / 3 (the face
// mean takes a third of each node), or kAttRef (negative; e never is) where
// the reference's expression has to run.  Within a source iteration the
// medium stays, so the factors can be stored by one sweep and read by the
// next ones.
constexpr double kAttRef = -1.0;

__device__ inline double node_att(const CellTerms& t, double s, const double* __restrict__ tab)
{
    const double x = t.ks * s;
    const int hx = __double2hiint(x);
    return (hx >= kFastXLo && hx <= kFastXHi) ? exp_neg(-x, tab) * (1.0 / 3.0) : kAttRef;
}

// A third of the node value from its factor e3 = e / 3 (s is read only on
// the reference's path; sr: the node's distance record), clamped at 0.
__device__ inline double node_third(const rts_medium& md, bool unit_i, const CellTerms& t, double e3,
                                    const double* sr, double I_0)
{
    const double I0 = unit_i ? I_0 : I_0 * md.i_scale;
    double I;
    if (__double2hiint(e3) >= 0) {
        // (e I0 + (1 - e) R/k) / 3, as R/3k + e/3 (I0 - R/k)
        I = fma(e3, I0 - t.Rk, t.Rk * (1.0 / 3.0));
    } else {
        const double s = *sr;
        I = node_illum_ref(md.mode, t.k, md.s_scale == 1.0 ? s : s * md.s_scale, I0, t.R) * (1.0 / 3.0);
    }
    if (__double2hiint(I) < 0) I = 0.0;  // I < 0 (the sign bit, tested as an integer)
    return unit_i ? I : I / md.i_scale;
}

// ReCalcIllum's term |old - cur| / cur for one face (Illum_async.cpp:488-493),
// folded into the running max.  The division runs only when the term can
// raise the max; NaN terms (0 / 0) drop out as in the reference.  (A screen
// of the terms on the exponent fields with integer operations, meant to spare
// the multiply and compare, measured 4-7 % slower: as compiled it added FP64
// operations instead of removing them.)
__device__ inline void norm_term(double old, double cur, double& loc)
{
    const double d = fabs(old - cur);
    if (d > loc * cur) {
        const double b = d / cur;
        if (b > loc) loc = b;
    }
}

__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// L2 eviction priorities of the sweep's loads.  Every direction reads the
// cells' neighbour table and medium entries (48 B per cell, 32 MB at 663,552
// cells: they fit in L2), while the items and attenuation factors (4 B and
// 24 B per item) are read once per sweep.  Loads of the shared tables are
// marked evict-last and the streams evict-first, so the streams do not push
// the tables out of L2 (cache hints only: the values are the same).
__device__ __forceinline__ uint64_t l2_policy_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t l2_policy_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ int4 ld_hint(const int4* q, uint64_t pol)
{
    int4 v;
    asm volatile("ld.global.nc.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(q), "l"(pol));
    return v;
}
__device__ __forceinline__ double2 ld_hint(const double2* q, uint64_t pol)
{
    double2 v;
    asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(q), "l"(pol));
    return v;
}
__device__ __forceinline__ double ld_hint(const double* q, uint64_t pol)
{
    double v;
    asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(q), "l"(pol));
    return v;
}
__device__ __forceinline__ uint32_t ld_hint(const uint32_t* q, uint64_t pol)
{
    uint32_t v;
    asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(q), "l"(pol));
    return v;
}

__device__ inline double pick(int g, double v0, double v1, double v2, double v3)
{
    return g == 0 ? v0 : g == 1 ? v1 : g == 2 ? v2 : v3;
}
__device__ inline int pick(int g, int v0, int v1, int v2, int v3)
{
    return g == 0 ? v0 : g == 1 ? v1 : g == 2 ? v2 : v3;
}

// One CTA per local direction.  First the boundary in-faces take their
// boundary value (BoundaryConditions: the node triple (I0, I0, I0)); then the
// steps of the dependency order in turn, a thread per out-face of the step:
// its cell's in-face means were written by upstream cells in earlier steps
// (visible after the barrier); it writes its mean to the face and to the
// neighbour's copy.  Every face is written once per sweep, so each writer
// takes ReCalcIllum's term against the old value.
// kAtt: 0 evaluates every node's attenuation factor, 1 also stores it,
// 2 reads the stored factors (no exponential).  kUnitI: i_scale == 1 (no
// scaling of the source and the node values, and the one-step face mean).
template <int kAtt, bool kUnitI>
__global__ void __launch_bounds__(SWEEP_THREADS, 7) sweep_kernel(SweepArgs a)
{
    const int64_t d = blockIdx.x;
    const int64_t N = a.N;
    const uint32_t* items = a.items[d];
    const double* recs = a.recs[d];
    const int32_t* steps = a.steps[d];
    const int ns = a.nsteps[d];
    const double* Sd = a.S + d * N;
    double* Il = a.illum + d * N * 4;
    const bool ball = a.md.radius > 0;
    constexpr bool unit_i = kUnitI;
    const bool unit_s = a.md.s_scale == 1.0;
    double* att = kAtt ? a.att[d] : nullptr;
    __shared__ double tab[kAtt == 2 ? 1 : kExpTable];
    if (kAtt != 2) {
        for (int i = threadIdx.x; i < kExpTable; i += SWEEP_THREADS) tab[i] = a.exp2tab[i];
        __syncthreads();
    }
    double loc = -1.0;
    {
        const uint32_t* bnd = a.bnd[d];
        const int nb = a.nbnd[d];
        for (int i = threadIdx.x; i < nb; i += SWEEP_THREADS) {
            const uint32_t id = bnd[i];
            const double I0 = a.bc[-a.pairs[id] - 1];
            const double mean = (I0 + I0 + I0) * (1.0 / 3.0);
            norm_term(Il[id], mean, loc);
            Il[id] = mean;
        }
    }
    const uint64_t keep = l2_policy_last(), stream = l2_policy_first();
    for (int L = 0; L < ns; ++L) {
        const int i1 = steps[L + 1];
        // the next item's word is loaded one iteration ahead and its cell's
        // rows prefetched into L1, so that the dependent loads of the next
        // iteration find them (the chain word -> cell -> rows otherwise
        // waits on memory twice per item)
        int i = steps[L] + threadIdx.x;
        uint32_t w_next = i < i1 ? ld_hint(items + i, stream) : 0u;
        for (; i < i1; i += SWEEP_THREADS) {
            const uint32_t w = w_next;
            if (i + SWEEP_THREADS < i1) {
                w_next = ld_hint(items + i + SWEEP_THREADS, stream);
                const int64_t cn = w_next >> 8;
                prefetch_l1(Il + 4 * cn);
                prefetch_l1(a.pairs + 4 * cn);
                prefetch_l1(a.med + 4 * cn);
                prefetch_l1(Sd + cn);
            }
            const int64_t c = w >> 8;
            const int f = (int)((w >> 6) & 3u);
            const double2 f01 = *reinterpret_cast<const double2*>(Il + 4 * c);
            const double2 f23 = *reinterpret_cast<const double2*>(Il + 4 * c + 2);
            const int4 pr = ld_hint(reinterpret_cast<const int4*>(a.pairs + 4 * c), keep);
            const double2 m01 = ld_hint(reinterpret_cast<const double2*>(a.med + 4 * c), keep);
            const double2 m23 = ld_hint(reinterpret_cast<const double2*>(a.med + 4 * c + 2), keep);
            const double Sc = Sd[c];
            const CellTerms cell = cell_terms(a.md, unit_i, unit_s, m01.x, m01.y, m23.x, m23.y, Sc);
            const double* sr = recs + 3 * (int64_t)i;
            double I0[3], e3[3];
            bool inb[3] = {false, false, false};
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                const int g = (int)((w >> (2 * m)) & 3u);
                const int nbg = pick(g, pr.x, pr.y, pr.z, pr.w);
                // CalculateIllumeOnInnerFace (Illum_async.cpp:172-199)
                I0[m] = nbg < 0 ? a.bc[-nbg - 1] : pick(g, f01.x, f01.y, f23.x, f23.y);
                if (ball) {  // class 0: other coefficients inside the ball
                    const double* x = a.nodes + 36 * c + 9 * f + 3 * m;
                    const double d0 = x[0] - a.md.ball[0], d1 = x[1] - a.md.ball[1], d2 = x[2] - a.md.ball[2];
                    inb[m] = sqrt(d0 * d0 + d1 * d1 + d2 * d2) < a.md.radius;
                }
                if (kAtt == 2) {
                    e3[m] = ld_hint(att + 3 * (int64_t)i + m, stream);
                } else {
                    const CellTerms t =
                        inb[m] ? cell_terms(a.md, unit_i, unit_s, a.ball[0], a.ball[1], a.ball[2], a.ball[3], Sc)
                               : cell;
                    e3[m] = node_att(t, sr[m], tab);
                    if (kAtt == 1) att[3 * (int64_t)i + m] = e3[m];
                }
            }
            // The face mean (I_0 + I_1 + I_2) / 3.  Where no node can clamp
            // (R/k >= 0, every I0 >= 0 and every factor on the fast form: each
            // node value R/k + e (I0 - R/k) is then >= 0, all sign bits tested
            // at once) it is R/k + sum_m e_m/3 (I0_m - R/k): 3 subtractions and
            // 3 FMAs instead of 6 operations for the nodes and 3 for the mean.
            double mean;
            if (unit_i && !ball &&
                (__double2hiint(e3[0]) | __double2hiint(e3[1]) | __double2hiint(e3[2]) | __double2hiint(I0[0]) |
                 __double2hiint(I0[1]) | __double2hiint(I0[2]) | __double2hiint(cell.Rk)) >= 0) {
                const double Rk = cell.Rk;
                mean = fma(e3[0], I0[0] - Rk, fma(e3[1], I0[1] - Rk, fma(e3[2], I0[2] - Rk, Rk)));
            } else {
                mean = 0.0;
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    const CellTerms t =
                        inb[m] ? cell_terms(a.md, unit_i, unit_s, a.ball[0], a.ball[1], a.ball[2], a.ball[3], Sc)
                               : cell;
                    mean += node_third(a.md, unit_i, t, e3[m], sr + m, I0[m]);
                }
            }
            const double old_f = pick(f, f01.x, f01.y, f23.x, f23.y);
            norm_term(old_f, mean, loc);
            Il[4 * c + f] = mean;
            const int nb = pick(f, pr.x, pr.y, pr.z, pr.w);
            if (nb >= 0) {
                // the neighbour's copy usually holds the value this face held
                // (both were written together by the last sweep): the same
                // term again, skipped after an integer compare of the bits
                const double old_n = Il[nb];
                if (__double_as_longlong(old_n) != __double_as_longlong(old_f)) norm_term(old_n, mean, loc);
                Il[nb] = mean;
            }
        }
        __syncthreads();
    }
    // max over the block, then over directions (non-negative doubles order
    // as their bit patterns; +1 keeps 0 for "no term")
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loc = fmax(loc, __shfl_xor_sync(0xffffffffu, loc, o));
    __shared__ double red[SWEEP_THREADS / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = red[0];
        for (int i = 1; i < SWEEP_THREADS / 32; ++i) m = fmax(m, red[i]);
        if (m >= 0) atomicMax(a.norm, (unsigned long long)__double_as_longlong(m) + 1ull);
    }
}

// ---------------------------------------------------------------- host side

void exp2_table(double* tab)
{
    for (int j = 0; j < kExpTable; ++j) tab[j] = exp2((double)j / kExpTable);
}

// exp_neg against CUDA's exp at n points spread over [-700, 0] (and the 1e-3
// end): the largest difference in units in the last place of CUDA's value.
__global__ void exp_check_kernel(int64_t n, const double* __restrict__ tab_in, double* out)
{
    __shared__ double tab[kExpTable];
    for (int i = threadIdx.x; i < kExpTable; i += blockDim.x) tab[i] = tab_in[i];
    __syncthreads();
    double worst = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double u = (double)i / (double)(n - 1);
        const double x = i & 1 ? -700.0 * u : -1e-3 - u * u;  // the whole range, and densely near 0
        const double a = exp_neg(x, tab), b = exp(x);
        const double ulp = fabs(__longlong_as_double(__double_as_longlong(b) + 1) - b);
        worst = fmax(worst, fabs(a - b) / ulp);
    }
    for (int o = 16; o > 0; o >>= 1) worst = fmax(worst, __shfl_xor_sync(0xffffffffu, worst, o));
    if ((threadIdx.x & 31) == 0) atomicMax((unsigned long long*)out, (unsigned long long)__double_as_longlong(worst));
}

int popcount4(int x) { return (x & 1) + ((x >> 1) & 1) + ((x >> 2) & 1) + ((x >> 3) & 1); }

// Dependency order of one direction: steps of cells whose in-faces all have
// known values (boundary faces are known from the start), each step in
// ascending cell id -- the order build_graph writes (build_graph/
// build_graph_calculation.cpp:347-391,482-510, driven by build_graph_main.cpp:
// 165-300).  A cell enters the step after the last of its upstream cells.
// lev receives the cell offset of every step and the end.  Returns false on
// a dependency cycle.
bool order_direction(int64_t N, const int32_t* pairs, const uint8_t* states, int32_t* order, std::vector<int32_t>& lev,
                     std::vector<int32_t>& indeg, std::vector<int32_t>& next)
{
    indeg.assign(N, 0);
    for (int64_t c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f)
            if (((states[c] >> f) & 1) && pairs[4 * c + f] >= 0) indeg[c]++;
    int64_t done = 0;
    lev.clear();
    for (int64_t c = 0; c < N; ++c)
        if (indeg[c] == 0) order[done++] = (int32_t)c;
    int64_t begin = 0;
    while (done > begin) {
        lev.push_back((int32_t)begin);
        const int64_t end = done;
        next.clear();
        for (int64_t i = begin; i < end; ++i) {
            const int64_t c = order[i];
            for (int f = 0; f < 4; ++f) {
                const int32_t nb = pairs[4 * c + f];
                if (nb < 0) continue;
                const int32_t nc = nb >> 2, nf = nb & 3;
                if (((states[nc] >> nf) & 1) && --indeg[nc] == 0) next.push_back(nc);
            }
        }
        std::sort(next.begin(), next.end());
        for (int32_t c : next) order[done++] = c;
        begin = end;
    }
    lev.push_back((int32_t)done);
    return done == N;
}

// Items, step offsets (in items) and boundary in-faces of one direction from
// its cell order, cell steps and face states.
void items_of(int64_t N, const int32_t* pairs, const uint8_t* states, const int32_t* order,
              const std::vector<int32_t>& lev, std::vector<uint32_t>& items, std::vector<int32_t>& steps,
              std::vector<uint32_t>& bnd)
{
    items.clear();
    steps.clear();
    bnd.clear();
    for (size_t L = 0; L + 1 < lev.size(); ++L) {
        steps.push_back((int32_t)items.size());
        for (int32_t p = lev[L]; p < lev[L + 1]; ++p) {
            const uint32_t c = (uint32_t)order[p];
            for (int f = 0; f < 4; ++f)
                if (!((states[c] >> f) & 1)) items.push_back(c << 8 | (uint32_t)f << 6);
        }
    }
    steps.push_back((int32_t)items.size());
    for (int64_t c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f)
            if (((states[c] >> f) & 1) && pairs[4 * c + f] < 0) bnd.push_back((uint32_t)(4 * c + f));
}

int alloc_tables(rts_ctx* ctx, rts_sweep_state& sw)
{
    const int64_t D = sw.D;
    void* p = nullptr;
    int rc;
    if ((rc = rts_dmalloc(ctx, &p, sizeof(uint32_t*) * D, "sweep item table")) != RTS_OK) return rc;
    sw.d_items = (uint32_t**)p;
    if ((rc = rts_dmalloc(ctx, &p, sizeof(double*) * D, "sweep record table")) != RTS_OK) return rc;
    sw.d_recs = (double**)p;
    if ((rc = rts_dmalloc(ctx, &p, sizeof(double*) * D, "sweep attenuation table")) != RTS_OK) return rc;
    sw.d_att = (double**)p;
    if ((rc = rts_dmalloc(ctx, &p, sizeof(int32_t*) * D, "sweep step table")) != RTS_OK) return rc;
    sw.d_steps = (int32_t**)p;
    if ((rc = rts_dmalloc(ctx, &p, sizeof(uint32_t*) * D, "sweep boundary table")) != RTS_OK) return rc;
    sw.d_bnd = (uint32_t**)p;
    if ((rc = rts_dmalloc(ctx, &p, rts_bytes<int32_t>(D), "sweep step counts")) != RTS_OK) return rc;
    sw.d_nsteps = (int32_t*)p;
    if ((rc = rts_dmalloc(ctx, &p, rts_bytes<int32_t>(D), "sweep boundary counts")) != RTS_OK) return rc;
    sw.d_nbnd = (int32_t*)p;
    sw.h_items.assign(D, nullptr);
    sw.h_recs.assign(D, nullptr);
    sw.h_att.assign(D, nullptr);
    sw.h_steps.assign(D, nullptr);
    sw.h_bnd.assign(D, nullptr);
    sw.h_nsteps.assign(D, 0);
    sw.h_nbnd.assign(D, 0);
    sw.h_nitems.assign(D, 0);
    sw.have.assign(D, 0);
    return RTS_OK;
}

void free_blocks(rts_ctx* ctx, rts_sweep_state& sw)
{
    for (auto& b : sw.blocks) rts_dfree(ctx, b.first, b.second);
    sw.blocks.clear();
    rts_dfree(ctx, sw.att_blk, sw.att_bytes);
    sw.att_blk = nullptr;
    sw.att_bytes = 0;
    sw.att_valid = false;
    std::fill(sw.h_items.begin(), sw.h_items.end(), nullptr);
    std::fill(sw.h_recs.begin(), sw.h_recs.end(), nullptr);
    std::fill(sw.h_steps.begin(), sw.h_steps.end(), nullptr);
    std::fill(sw.h_bnd.begin(), sw.h_bnd.end(), nullptr);
    std::fill(sw.h_nsteps.begin(), sw.h_nsteps.end(), 0);
    std::fill(sw.h_nbnd.begin(), sw.h_nbnd.end(), 0);
    std::fill(sw.h_nitems.begin(), sw.h_nitems.end(), 0);
    std::fill(sw.have.begin(), sw.have.end(), 0);
    sw.records = sw.max_levels = 0;
}

int alloc_block(rts_ctx* ctx, rts_sweep_state& sw, void** p, size_t bytes, const char* what)
{
    bytes = std::max<size_t>(bytes, 16);
    int rc = rts_dmalloc(ctx, p, bytes, what);
    if (rc == RTS_OK) sw.blocks.push_back({*p, bytes});
    return rc;
}

int upload_tables(rts_ctx* ctx, rts_sweep_state& sw, cudaStream_t st)
{
    const int64_t D = sw.D;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.d_items, sw.h_items.data(), sizeof(uint32_t*) * D, cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.d_recs, sw.h_recs.data(), sizeof(double*) * D, cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.d_steps, sw.h_steps.data(), sizeof(int32_t*) * D, cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.d_bnd, sw.h_bnd.data(), sizeof(uint32_t*) * D, cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.d_nsteps, sw.h_nsteps.data(), sizeof(int32_t) * D, cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.d_nbnd, sw.h_nbnd.data(), sizeof(int32_t) * D, cudaMemcpyHostToDevice, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // pageable sources
    return RTS_OK;
}

int check_flag(rts_ctx* ctx, const char* what)
{
    int flag = 0;
    RTS_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag + 2, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        cudaMemset(ctx->d_flag + 2, 0, sizeof(int));
        return rts_fail(ctx, RTS_ERR_UNSUPPORTED, "%s: an out-face node found no in-face (a direction parallel to a face)",
                        what);
    }
    return RTS_OK;
}

}  // namespace

void rts_sweep_free(rts_ctx* ctx)
{
    rts_sweep_state* sw = ctx->sweep;
    if (!sw) return;
    free_blocks(ctx, *sw);
    const int64_t N = sw->N, D = sw->D;
    rts_dfree(ctx, sw->d_vert, rts_bytes<double>(N * 12));
    rts_dfree(ctx, sw->d_pairs, rts_bytes<int32_t>(N * 4));
    rts_dfree(ctx, sw->d_normals, rts_bytes<double>(N * 12));
    rts_dfree(ctx, sw->d_nodes, rts_bytes<double>(N * 36));
    rts_dfree(ctx, sw->d_med, rts_bytes<double>(N * 4));
    rts_dfree(ctx, sw->d_norm, sizeof(unsigned long long));
    rts_dfree(ctx, sw->d_items, sizeof(uint32_t*) * D);
    rts_dfree(ctx, sw->d_recs, sizeof(double*) * D);
    rts_dfree(ctx, sw->d_att, sizeof(double*) * D);
    rts_dfree(ctx, sw->d_steps, sizeof(int32_t*) * D);
    rts_dfree(ctx, sw->d_bnd, sizeof(uint32_t*) * D);
    rts_dfree(ctx, sw->d_nsteps, rts_bytes<int32_t>(D));
    rts_dfree(ctx, sw->d_nbnd, rts_bytes<int32_t>(D));
    delete sw;
    ctx->sweep = nullptr;
}

extern "C" int rts_sweep_set_mesh(rts_ctx* ctx, const double* vert, const int32_t* pairs, const double* normals)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->d_illum, RTS_ERR_BAD_STATE, "rts_sweep_set_mesh before rts_init");
    RTS_REQUIRE(ctx, vert && pairs && normals, RTS_ERR_INVALID_ARGUMENT, "rts_sweep_set_mesh: null array");
    const int64_t N = ctx->N;
    RTS_REQUIRE(ctx, N < (int64_t)1 << 24, RTS_ERR_INVALID_ARGUMENT,
                "rts_sweep_set_mesh: %lld cells; the sweep packs cell ids in 24 bits", (long long)N);
    for (int64_t i = 0; i < 4 * N; ++i)
        RTS_REQUIRE(ctx, pairs[i] < 4 * N && pairs[i] >= RTS_BOUND_INNER, RTS_ERR_INVALID_ARGUMENT,
                    "rts_sweep_set_mesh: pairs[%lld] = %d is neither a face nor a boundary code", (long long)i,
                    (int)pairs[i]);
    rts_sweep_free(ctx);
    rts_sweep_state* sw = new rts_sweep_state();
    ctx->sweep = sw;
    sw->N = N;
    sw->D = ctx->local();
    sw->h_vert.assign(vert, vert + 12 * N);
    sw->h_pairs.assign(pairs, pairs + 4 * N);
    sw->h_normals.assign(normals, normals + 12 * N);
    std::vector<double> nodes(36 * N);
    rts_sweep_nodes_host(N, vert, nodes.data());
    void* p = nullptr;
    int rc;
    if ((rc = rts_dmalloc(ctx, &p, rts_bytes<double>(N * 12), "sweep vertices")) != RTS_OK) return rc;
    sw->d_vert = (double*)p;
    if ((rc = rts_dmalloc(ctx, &p, rts_bytes<int32_t>(N * 4), "sweep pairs")) != RTS_OK) return rc;
    sw->d_pairs = (int32_t*)p;
    if ((rc = rts_dmalloc(ctx, &p, rts_bytes<double>(N * 12), "sweep normals")) != RTS_OK) return rc;
    sw->d_normals = (double*)p;
    if ((rc = rts_dmalloc(ctx, &p, rts_bytes<double>(N * 36), "sweep nodes")) != RTS_OK) return rc;
    sw->d_nodes = (double*)p;
    if ((rc = rts_dmalloc(ctx, &p, rts_bytes<double>(N * 4), "sweep medium")) != RTS_OK) return rc;
    sw->d_med = (double*)p;
    if ((rc = rts_dmalloc(ctx, &p, sizeof(unsigned long long), "sweep norm")) != RTS_OK) return rc;
    sw->d_norm = (unsigned long long*)p;
    RTS_CUDA_TRY(ctx, cudaMemcpy(sw->d_vert, vert, rts_bytes<double>(N * 12), cudaMemcpyHostToDevice));
    RTS_CUDA_TRY(ctx, cudaMemcpy(sw->d_pairs, pairs, rts_bytes<int32_t>(N * 4), cudaMemcpyHostToDevice));
    RTS_CUDA_TRY(ctx, cudaMemcpy(sw->d_normals, normals, rts_bytes<double>(N * 12), cudaMemcpyHostToDevice));
    RTS_CUDA_TRY(ctx, cudaMemcpy(sw->d_nodes, nodes.data(), rts_bytes<double>(N * 36), cudaMemcpyHostToDevice));
    RTS_CUDA_TRY(ctx, cudaMemset(sw->d_med, 0, rts_bytes<double>(N * 4)));
    return alloc_tables(ctx, *sw);
}

extern "C" int rts_sweep_build(rts_ctx* ctx, int64_t* records, int64_t* levels)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->sweep, RTS_ERR_BAD_STATE, "rts_sweep_build before rts_sweep_set_mesh");
    rts_sweep_state& sw = *ctx->sweep;
    const int64_t N = sw.N, D = sw.D;
    free_blocks(ctx, sw);
    // host: face states, dependency order, items of every direction
    std::vector<uint8_t> states((size_t)(D * N));
    std::vector<std::vector<uint32_t>> items((size_t)D), bnd((size_t)D);
    std::vector<std::vector<int32_t>> steps((size_t)D);
    std::vector<char> bad((size_t)D, 0);
    const int nthr = (int)std::max<int64_t>(1, std::min<int64_t>(D, std::max(1u, std::thread::hardware_concurrency())));
    auto work = [&](int w) {
        std::vector<int32_t> order((size_t)N), lev, indeg, next;
        for (int64_t d = w; d < D; d += nthr) {
            const double* dir = ctx->h_xyz.data() + 3 * (ctx->out_start + d);
            uint8_t* st = states.data() + d * N;
            for (int64_t c = 0; c < N; ++c) {
                int s = 0;
                const double* n = sw.h_normals.data() + 12 * c;
                for (int f = 0; f < 4; ++f)
                    if (n[3 * f] * dir[0] + n[3 * f + 1] * dir[1] + n[3 * f + 2] * dir[2] < -SWEEP_EPS) s |= 1 << f;
                st[c] = (uint8_t)s;
            }
            if (!order_direction(N, sw.h_pairs.data(), st, order.data(), lev, indeg, next)) {
                bad[d] = 1;
                continue;
            }
            items_of(N, sw.h_pairs.data(), st, order.data(), lev, items[d], steps[d], bnd[d]);
        }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < nthr; ++w) pool.emplace_back(work, w);
    work(0);
    for (auto& t : pool) t.join();
    for (int64_t d = 0; d < D; ++d)
        RTS_REQUIRE(ctx, !bad[d], RTS_ERR_UNSUPPORTED, "rts_sweep_build: direction %lld has a dependency cycle",
                    (long long)(ctx->out_start + d));
    // device: one block each of items, node records, steps and boundary faces
    int64_t ni = 0, nl = 0, nbd = 0, maxl = 0;
    for (int64_t d = 0; d < D; ++d) {
        ni += (int64_t)items[d].size();
        nl += (int64_t)steps[d].size();
        nbd += (int64_t)bnd[d].size();
        maxl = std::max<int64_t>(maxl, (int64_t)steps[d].size() - 1);
    }
    void *iblk = nullptr, *rblk = nullptr, *lblk = nullptr, *bblk = nullptr, *sblk = nullptr;
    int rc;
    if ((rc = alloc_block(ctx, sw, &iblk, rts_bytes<uint32_t>(ni), "sweep items")) != RTS_OK) return rc;
    if ((rc = alloc_block(ctx, sw, &rblk, rts_bytes<double>(3 * ni), "sweep node records")) != RTS_OK) return rc;
    if ((rc = alloc_block(ctx, sw, &lblk, rts_bytes<int32_t>(nl), "sweep steps")) != RTS_OK) return rc;
    if ((rc = alloc_block(ctx, sw, &bblk, rts_bytes<uint32_t>(nbd), "sweep boundary faces")) != RTS_OK) return rc;
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    int64_t io = 0, lo = 0, bo = 0;
    for (int64_t d = 0; d < D; ++d) {
        sw.h_items[d] = (uint32_t*)iblk + io;
        sw.h_recs[d] = (double*)rblk + 3 * io;
        sw.h_steps[d] = (int32_t*)lblk + lo;
        sw.h_bnd[d] = (uint32_t*)bblk + bo;
        sw.h_nsteps[d] = (int32_t)steps[d].size() - 1;
        sw.h_nbnd[d] = (int32_t)bnd[d].size();
        sw.h_nitems[d] = (int64_t)items[d].size();
        RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.h_items[d], items[d].data(), rts_bytes<uint32_t>(items[d].size()),
                                          cudaMemcpyHostToDevice, st));
        RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.h_steps[d], steps[d].data(), rts_bytes<int32_t>(steps[d].size()),
                                          cudaMemcpyHostToDevice, st));
        if (!bnd[d].empty())
            RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.h_bnd[d], bnd[d].data(), rts_bytes<uint32_t>(bnd[d].size()),
                                              cudaMemcpyHostToDevice, st));
        io += (int64_t)items[d].size();
        lo += (int64_t)steps[d].size();
        bo += (int64_t)bnd[d].size();
    }
    // the face states, for the builder kernel only
    if ((rc = rts_dmalloc(ctx, &sblk, rts_bytes<uint8_t>(std::max<int64_t>(D * N, 16)), "sweep face states")) !=
        RTS_OK)
        return rc;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sblk, states.data(), rts_bytes<uint8_t>(D * N), cudaMemcpyHostToDevice, st));
    if ((rc = upload_tables(ctx, sw, st)) != RTS_OK) {
        rts_dfree(ctx, sblk, rts_bytes<uint8_t>(std::max<int64_t>(D * N, 16)));
        return rc;
    }
    // device: the in-face frames, then the in-face and distance of every node
    void* fblk = nullptr;
    if ((rc = rts_dmalloc(ctx, &fblk, rts_bytes<double>(kFrame * 4 * N), "sweep face frames")) != RTS_OK) {
        rts_dfree(ctx, sblk, rts_bytes<uint8_t>(std::max<int64_t>(D * N, 16)));
        return rc;
    }
    if (N > 0) {
        sweep_frames_kernel<<<(unsigned)std::min<int64_t>((4 * N + 255) / 256, 8192), 256, 0, st>>>(
            sw.d_vert, sw.d_normals, N, (double*)fblk);
        ctx->launches++;
    }
    X0Args a;
    a.vert = sw.d_vert;
    a.frames = (const double*)fblk;
    a.nodes = sw.d_nodes;
    a.dirs = ctx->d_xyz + 3 * ctx->out_start;
    a.states = (const uint8_t*)sblk;
    a.items = sw.d_items;
    a.recs = sw.d_recs;
    a.steps = sw.d_steps;
    a.nsteps = sw.d_nsteps;
    a.N = N;
    a.flag = ctx->d_flag + 2;
    if (D > 0) {
        const int64_t per = std::max<int64_t>(1, std::min<int64_t>((2 * N + 255) / 256, 64));
        cudaError_t e = cudaSuccess;
        for (int64_t d0 = 0; d0 < D && e == cudaSuccess; d0 += 65535) {
            a.d0 = d0;
            sweep_x0_kernel<<<dim3((unsigned)per, (unsigned)std::min<int64_t>(D - d0, 65535)), 256, 0, st>>>(a);
            e = cudaGetLastError();
            ctx->launches++;
        }
        cudaStreamSynchronize(st);
        rts_dfree(ctx, sblk, rts_bytes<uint8_t>(std::max<int64_t>(D * N, 16)));
        rts_dfree(ctx, fblk, rts_bytes<double>(kFrame * 4 * N));
        if (e != cudaSuccess)
            return rts_fail(ctx, RTS_ERR_CUDA, "launch of sweep_x0_kernel failed: %s", cudaGetErrorString(e));
    } else {
        rts_dfree(ctx, sblk, rts_bytes<uint8_t>(16));
        rts_dfree(ctx, fblk, rts_bytes<double>(kFrame * 4 * N));
    }
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if ((rc = check_flag(ctx, "rts_sweep_build")) != RTS_OK) return rc;
    std::fill(sw.have.begin(), sw.have.end(), 1);
    sw.records = 3 * ni;
    sw.max_levels = maxl;
    if (records) *records = 3 * ni;
    if (levels) *levels = maxl;
    return RTS_OK;
}

extern "C" int rts_sweep_import_direction(rts_ctx* ctx, int64_t d, const int32_t* order, const int32_t* states,
                                          const void* locx0, int64_t count)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->sweep, RTS_ERR_BAD_STATE, "rts_sweep_import_direction before rts_sweep_set_mesh");
    rts_sweep_state& sw = *ctx->sweep;
    const int64_t N = sw.N;
    RTS_REQUIRE(ctx, 0 <= d && d < sw.D, RTS_ERR_INVALID_ARGUMENT, "rts_sweep_import_direction: direction %lld outside "
                "the %lld local directions", (long long)d, (long long)sw.D);
    RTS_REQUIRE(ctx, order && states && (locx0 || count == 0), RTS_ERR_INVALID_ARGUMENT,
                "rts_sweep_import_direction: null array");
    const int32_t* pairs = sw.h_pairs.data();
    // steps from the file's order: a cell goes one step after its latest
    // upstream cell (the file's order must list upstream cells first)
    std::vector<int32_t> step((size_t)N, -1), start_rec((size_t)N, 0);
    std::vector<uint8_t> st8((size_t)N);
    int64_t rec = 0;
    int32_t nsteps = 0;
    for (int64_t h = 0; h < N; ++h) {
        const int32_t c = order[h];
        RTS_REQUIRE(ctx, 0 <= c && c < N && step[c] < 0, RTS_ERR_INVALID_ARGUMENT,
                    "rts_sweep_import_direction: order[%lld] = %d is not a new cell", (long long)h, (int)c);
        const int st = states[c] & 15;
        st8[c] = (uint8_t)st;
        int32_t lv = 0;
        for (int f = 0; f < 4; ++f) {
            if (!((st >> f) & 1) || pairs[4 * c + f] < 0) continue;
            const int32_t u = pairs[4 * c + f] >> 2;
            RTS_REQUIRE(ctx, step[u] >= 0, RTS_ERR_INVALID_ARGUMENT,
                        "rts_sweep_import_direction: cell %d comes before its upstream cell %d", (int)c, (int)u);
            lv = std::max(lv, step[u] + 1);
        }
        step[c] = lv;
        nsteps = std::max(nsteps, lv + 1);
        start_rec[c] = (int32_t)rec;
        rec += 3 * (4 - popcount4(st));
    }
    RTS_REQUIRE(ctx, rec == count, RTS_ERR_INVALID_ARGUMENT,
                "rts_sweep_import_direction: %lld records given, the states need %lld", (long long)count,
                (long long)rec);
    // cells grouped by step, the file's order kept within a step
    std::vector<int32_t> lev((size_t)nsteps + 1, 0), pos_order((size_t)N);
    for (int64_t c = 0; c < N; ++c) lev[step[c] + 1]++;
    for (int32_t L = 0; L < nsteps; ++L) lev[L + 1] += lev[L];
    {
        std::vector<int32_t> fill(lev.begin(), lev.end() - 1);
        for (int64_t h = 0; h < N; ++h) pos_order[fill[step[order[h]]]++] = order[h];
    }
    std::vector<uint32_t> items, bnd;
    std::vector<int32_t> steps;
    items_of(N, pairs, st8.data(), pos_order.data(), lev, items, steps, bnd);
    // node records of every item, in item order
    std::vector<double> recs(std::max<size_t>(3 * items.size(), 1));
    const unsigned char* in = (const unsigned char*)locx0;
    for (size_t i = 0; i < items.size(); ++i) {
        const uint32_t c = items[i] >> 8;
        const int f = (int)((items[i] >> 6) & 3u);
        const int st = st8[c];
        int slot = 0;  // rank of f among the cell's out-faces
        for (int g = 0; g < f; ++g)
            if (!((st >> g) & 1)) ++slot;
        for (int m = 0; m < 3; ++m) {
            const unsigned char* r = in + 32 * (int64_t)(start_rec[c] + 3 * slot + m);
            double sv;
            memcpy(&sv, r, sizeof(double));
            const int g = r[24];
            RTS_REQUIRE(ctx, g < 4 && ((st >> g) & 1), RTS_ERR_INVALID_ARGUMENT,
                        "rts_sweep_import_direction: record %lld names face %d, not an in-face of cell %u",
                        (long long)(start_rec[c] + 3 * slot + m), g, c);
            recs[3 * i + m] = sv;
            items[i] |= (uint32_t)g << (2 * m);
        }
    }
    // this direction's own blocks
    int rc;
    void *iblk = nullptr, *rblk = nullptr, *lblk = nullptr, *bblk = nullptr;
    if ((rc = alloc_block(ctx, sw, &iblk, rts_bytes<uint32_t>(items.size()), "sweep items")) != RTS_OK) return rc;
    if ((rc = alloc_block(ctx, sw, &rblk, rts_bytes<double>(3 * items.size()), "sweep node records")) != RTS_OK)
        return rc;
    if ((rc = alloc_block(ctx, sw, &lblk, rts_bytes<int32_t>(steps.size()), "sweep steps")) != RTS_OK) return rc;
    if ((rc = alloc_block(ctx, sw, &bblk, rts_bytes<uint32_t>(bnd.size()), "sweep boundary faces")) != RTS_OK)
        return rc;
    RTS_CUDA_TRY(ctx, cudaMemcpy(iblk, items.data(), rts_bytes<uint32_t>(items.size()), cudaMemcpyHostToDevice));
    RTS_CUDA_TRY(ctx, cudaMemcpy(rblk, recs.data(), rts_bytes<double>(3 * items.size()), cudaMemcpyHostToDevice));
    RTS_CUDA_TRY(ctx, cudaMemcpy(lblk, steps.data(), rts_bytes<int32_t>(steps.size()), cudaMemcpyHostToDevice));
    if (!bnd.empty())
        RTS_CUDA_TRY(ctx, cudaMemcpy(bblk, bnd.data(), rts_bytes<uint32_t>(bnd.size()), cudaMemcpyHostToDevice));
    sw.att_valid = false;
    if (sw.have[d]) sw.records -= 3 * sw.h_nitems[d];
    sw.records += 3 * (int64_t)items.size();
    sw.h_items[d] = (uint32_t*)iblk;
    sw.h_recs[d] = (double*)rblk;
    sw.h_steps[d] = (int32_t*)lblk;
    sw.h_bnd[d] = (uint32_t*)bblk;
    sw.h_nsteps[d] = nsteps;
    sw.h_nbnd[d] = (int32_t)bnd.size();
    sw.h_nitems[d] = (int64_t)items.size();
    sw.have[d] = 1;
    sw.max_levels = std::max<int64_t>(sw.max_levels, nsteps);
    return upload_tables(ctx, sw, ctx->streams[RTS_STREAM_SCATTERING_1]);
}

extern "C" int rts_sweep_export_direction(rts_ctx* ctx, int64_t d, int32_t* order, int32_t* states, void* locx0,
                                          int64_t capacity, int64_t* count)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->sweep, RTS_ERR_BAD_STATE, "rts_sweep_export_direction before rts_sweep_set_mesh");
    rts_sweep_state& sw = *ctx->sweep;
    const int64_t N = sw.N;
    RTS_REQUIRE(ctx, 0 <= d && d < sw.D && sw.have[d], RTS_ERR_INVALID_ARGUMENT,
                "rts_sweep_export_direction: direction %lld has no structures", (long long)d);
    const int64_t ni = sw.h_nitems[d];
    if (count) *count = 3 * ni;
    std::vector<uint32_t> items((size_t)std::max<int64_t>(ni, 1));
    if (ni)
        RTS_CUDA_TRY(ctx, cudaMemcpy(items.data(), sw.h_items[d], rts_bytes<uint32_t>(ni), cudaMemcpyDeviceToHost));
    // cells in order of their first item; a cell's faces that are not items are in-faces
    std::vector<int32_t> od;
    std::vector<uint8_t> outs((size_t)N, 0);
    od.reserve((size_t)N);
    for (int64_t i = 0; i < ni; ++i) {
        const uint32_t c = items[i] >> 8;
        if (!outs[c]) od.push_back((int32_t)c);
        outs[c] |= (uint8_t)(1u << ((items[i] >> 6) & 3u));
    }
    RTS_REQUIRE(ctx, (int64_t)od.size() == N, RTS_ERR_BAD_STATE,
                "rts_sweep_export_direction: %lld of %lld cells have out-faces", (long long)od.size(), (long long)N);
    if (order) memcpy(order, od.data(), rts_bytes<int32_t>(N));
    if (states)
        for (int64_t c = 0; c < N; ++c) states[c] = (int32_t)(~outs[c] & 15u);
    if (!locx0 || capacity < 3 * ni) return RTS_OK;
    std::vector<double> recs((size_t)std::max<int64_t>(3 * ni, 1));
    if (ni)
        RTS_CUDA_TRY(ctx, cudaMemcpy(recs.data(), sw.h_recs[d], rts_bytes<double>(3 * ni), cudaMemcpyDeviceToHost));
    unsigned char* out = (unsigned char*)locx0;
    memset(out, 0, (size_t)(32 * 3 * ni));
    for (int64_t i = 0; i < 3 * ni; ++i) {
        memcpy(out + 32 * i, &recs[i], sizeof(double));
        out[32 * i + 24] = (unsigned char)((items[i / 3] >> (2 * (i % 3))) & 3u);
    }
    return RTS_OK;
}

extern "C" int rts_sweep_set_medium(rts_ctx* ctx, const rts_medium* md, const double* alpha, const double* beta,
                                    const double* Q, const double* bc)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, ctx->sweep, RTS_ERR_BAD_STATE, "rts_sweep_set_medium before rts_sweep_set_mesh");
    RTS_REQUIRE(ctx, md && alpha && beta && Q, RTS_ERR_INVALID_ARGUMENT, "rts_sweep_set_medium: null argument");
    RTS_REQUIRE(ctx, md->mode == RTS_MEDIUM_SCATTERING || md->mode == RTS_MEDIUM_ABSORPTION, RTS_ERR_INVALID_ARGUMENT,
                "rts_sweep_set_medium: unknown mode %d", md->mode);
    RTS_REQUIRE(ctx, md->i_scale != 0.0, RTS_ERR_INVALID_ARGUMENT, "rts_sweep_set_medium: i_scale must not be 0");
    rts_sweep_state& sw = *ctx->sweep;
    const int64_t N = sw.N;
    std::vector<double> m((size_t)(4 * N));
    for (int64_t c = 0; c < N; ++c) medium_entry(md->mode, alpha[c], beta[c], Q[c], &m[4 * c]);
    RTS_CUDA_TRY(ctx, cudaMemcpy(sw.d_med, m.data(), rts_bytes<double>(4 * N), cudaMemcpyHostToDevice));
    sw.md = *md;
    if (bc)
        for (int i = 0; i < 4; ++i) sw.bc[i] = bc[i];
    else
        sw.bc[0] = 0.0, sw.bc[1] = 0.0, sw.bc[2] = 1.0, sw.bc[3] = 0.0;
    sw.has_medium = true;
    sw.att_valid = false;
    return RTS_OK;
}

// The form of the next sweep: 2 reads the stored attenuation factors, 1
// stores them (laying out, and where needed allocating, their block), 0
// evaluates them (the cache switched off, or no room for the factors).
static int att_mode(rts_ctx* ctx, rts_sweep_state& sw, cudaStream_t st, int* mode)
{
    *mode = 0;
    if (!ctx->sweep_cache) return RTS_OK;
    if (sw.att_valid) {
        *mode = 2;
        return RTS_OK;
    }
    int64_t nrec = 0;
    for (int64_t d = 0; d < sw.D; ++d) nrec += 3 * sw.h_nitems[d];
    const size_t need = rts_bytes<double>(std::max<int64_t>(nrec, 2));
    if (sw.att_bytes != need) {
        rts_dfree(ctx, sw.att_blk, sw.att_bytes);
        sw.att_blk = nullptr;
        sw.att_bytes = 0;
        const std::string keep = ctx->last_error;
        void* p = nullptr;
        if (rts_dmalloc(ctx, &p, need, "sweep attenuation factors") != RTS_OK) {
            ctx->last_error = keep;  // not an error: this sweep evaluates the factors
            return RTS_OK;
        }
        sw.att_blk = (double*)p;
        sw.att_bytes = need;
    }
    int64_t o = 0;
    for (int64_t d = 0; d < sw.D; ++d) {
        sw.h_att[d] = sw.att_blk + o;
        o += 3 * sw.h_nitems[d];
    }
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(sw.d_att, sw.h_att.data(), sizeof(double*) * sw.D, cudaMemcpyHostToDevice, st));
    *mode = 1;
    return RTS_OK;
}

static int enqueue_sweep(rts_ctx* ctx, cudaStream_t st)
{
    rts_sweep_state& sw = *ctx->sweep;
    int mode = 0;
    int rc = att_mode(ctx, sw, st, &mode);
    if (rc != RTS_OK) return rc;
    RTS_CUDA_TRY(ctx, cudaMemsetAsync(sw.d_norm, 0, sizeof(unsigned long long), st));
    SweepArgs a;
    a.items = sw.d_items;
    a.recs = sw.d_recs;
    a.att = sw.d_att;
    a.steps = sw.d_steps;
    a.bnd = sw.d_bnd;
    a.nsteps = sw.d_nsteps;
    a.nbnd = sw.d_nbnd;
    a.pairs = sw.d_pairs;
    a.nodes = sw.d_nodes;
    a.med = sw.d_med;
    a.S = ctx->d_S;
    a.illum = ctx->d_illum + ctx->out_start * sw.N * 4;
    a.N = sw.N;
    a.md = sw.md;
    for (int i = 0; i < 4; ++i) a.bc[i] = sw.bc[i];
    exp2_table(a.exp2tab);
    medium_entry(sw.md.mode, sw.md.ball_alpha, sw.md.ball_beta, sw.md.ball_q, a.ball);
    a.norm = sw.d_norm;
    if (sw.D > 0) {
        rts_timing_begin(ctx, st);
        const dim3 grid((unsigned)sw.D);
        if (sw.md.i_scale == 1.0) {
            if (mode == 2)
                sweep_kernel<2, true><<<grid, SWEEP_THREADS, 0, st>>>(a);
            else if (mode == 1)
                sweep_kernel<1, true><<<grid, SWEEP_THREADS, 0, st>>>(a);
            else
                sweep_kernel<0, true><<<grid, SWEEP_THREADS, 0, st>>>(a);
        } else {
            if (mode == 2)
                sweep_kernel<2, false><<<grid, SWEEP_THREADS, 0, st>>>(a);
            else if (mode == 1)
                sweep_kernel<1, false><<<grid, SWEEP_THREADS, 0, st>>>(a);
            else
                sweep_kernel<0, false><<<grid, SWEEP_THREADS, 0, st>>>(a);
        }
        rts_timing_end(ctx, st);
        RTS_CHECK_LAUNCH(ctx, "sweep_kernel");
        ctx->launches++;
        if (mode == 1) sw.att_valid = true;
    }
    return RTS_OK;
}

static int read_norm(rts_ctx* ctx, cudaStream_t st, double* norm)
{
    unsigned long long bits = 0;
    RTS_CUDA_TRY(ctx, cudaMemcpyAsync(&bits, ctx->sweep->d_norm, sizeof(bits), cudaMemcpyDeviceToHost, st));
    RTS_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if (bits == 0) {
        *norm = -1.0;
    } else {
        const unsigned long long b = bits - 1;
        memcpy(norm, &b, sizeof(double));
    }
    return RTS_OK;
}

static int sweep_ready(rts_ctx* ctx)
{
    RTS_REQUIRE(ctx, ctx->sweep, RTS_ERR_BAD_STATE, "sweep before rts_sweep_set_mesh");
    rts_sweep_state& sw = *ctx->sweep;
    RTS_REQUIRE(ctx, sw.has_medium, RTS_ERR_BAD_STATE, "sweep before rts_sweep_set_medium");
    for (int64_t d = 0; d < sw.D; ++d)
        RTS_REQUIRE(ctx, sw.have[d], RTS_ERR_BAD_STATE,
                    "sweep: direction %lld has no structures (rts_sweep_build or rts_sweep_import_direction)",
                    (long long)d);
    return RTS_OK;
}

extern "C" int rts_sweep(rts_ctx* ctx, int stream, double* norm)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, stream >= 0 && stream < RTS_STREAM_COUNT, RTS_ERR_INVALID_ARGUMENT, "bad stream id %d", stream);
    int rc = sweep_ready(ctx);
    if (rc != RTS_OK) return rc;
    cudaStream_t st = ctx->streams[stream];
    rts_inputs_changed(ctx);  // the device Illum changes under a resident tensor-core iteration
    if ((rc = enqueue_sweep(ctx, st)) != RTS_OK) return rc;
    if (norm) return read_norm(ctx, st, norm);
    return RTS_OK;
}

extern "C" int rts_illum_solve(rts_ctx* ctx, int precision, int max_iter, double accuracy, int64_t* iters,
                               double* norms)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, max_iter >= 1, RTS_ERR_INVALID_ARGUMENT, "rts_illum_solve: max_iter %d < 1", max_iter);
    const bool tensor =
        precision == RTS_PREC_BF16X3 || precision == RTS_PREC_FP16X3 || precision == RTS_PREC_TF32X3;
    RTS_REQUIRE(ctx, tensor || precision == RTS_PREC_FP64, RTS_ERR_INVALID_ARGUMENT, "unknown precision %d",
                precision);
    int rc = sweep_ready(ctx);
    if (rc != RTS_OK) return rc;
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    rts_inputs_changed(ctx);
    int64_t count = 0;
    double norm = -1.0;
    do {
        if ((rc = enqueue_sweep(ctx, st)) != RTS_OK) return rc;
        if (max_iter > 1) {
            rc = tensor ? rts_split_device_call(ctx, precision, st)
                        : rts_launch_scatter_fp64(ctx, 0, ctx->local(), st, nullptr, 0.0, false, false);
            if (rc != RTS_OK) return rc;
        }
        if ((rc = read_norm(ctx, st, &norm)) != RTS_OK) return rc;
        if (norms) norms[count] = norm;
        ++count;
    } while (norm > accuracy && count < max_iter);
    if (iters) *iters = count;
    if (tensor) {
        int flag = 0;
        RTS_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
        if (flag) return rts_fail(ctx, RTS_ERR_DEVICE_WAIT, "tensor-path kernel reported device flag %d", flag);
    }
    return RTS_OK;
}

extern "C" int rts_sweep_exp_check(rts_ctx* ctx, int64_t n, double* max_ulp)
{
    if (!ctx) return RTS_ERR_INVALID_ARGUMENT;
    RTS_REQUIRE(ctx, n >= 2 && max_ulp, RTS_ERR_INVALID_ARGUMENT, "rts_sweep_exp_check: n >= 2 and an output");
    double tab[kExpTable];
    exp2_table(tab);
    void* p = nullptr;
    int rc = rts_dmalloc(ctx, &p, (kExpTable + 1) * sizeof(double), "exp check");
    if (rc != RTS_OK) return rc;
    double* d = (double*)p;
    cudaStream_t st = ctx->streams[RTS_STREAM_SCATTERING_1];
    cudaError_t e = cudaMemcpyAsync(d, tab, kExpTable * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d + kExpTable, 0, sizeof(double), st);
    if (e == cudaSuccess) {
        exp_check_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, 0, st>>>(n, d, d + kExpTable);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(max_ulp, d + kExpTable, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    rts_dfree(ctx, d, (kExpTable + 1) * sizeof(double));
    if (e != cudaSuccess) return rts_fail(ctx, RTS_ERR_CUDA, "rts_sweep_exp_check: %s", cudaGetErrorString(e));
    ctx->launches++;
    return RTS_OK;
}

// The reference's unit system and constants (global_value.h:32-52): code units
// of length, density, pressure and radiation, and SI physical constants.
namespace gas {
constexpr double kPi = 3.14159265358979323846;
constexpr double kCLight = 299792458.0;
constexpr double kDist = 1e6;
constexpr double kVelocity = 3 * 1e8;
constexpr double kDensity = 3.34 * 10e-14;
constexpr double kPressure = kDensity * kVelocity * kVelocity;
constexpr double kRadiation = kDensity * kVelocity * kVelocity * kVelocity;
constexpr double kRGas = 8.314;
constexpr double kHPlank = 6.62 * 1e-34;
constexpr double kBoltzmann = 1.38 * 1e-23;
constexpr double kSigmaThomson = 6.652 * 1e-29;
constexpr double kMHydrogen = 1.6735575 * 1e-27;
}  // namespace gas

extern "C" int rts_sweep_medium_gas(int64_t N, const double* density, const double* pressure, double* alpha,
                                    double* beta, double* Q, rts_medium* md)
{
    if (N < 0 || (N > 0 && (!density || !pressure || !alpha || !beta || !Q)) || !md) return RTS_ERR_INVALID_ARGUMENT;
    using namespace gas;
    for (int64_t c = 0; c < N; ++c) {
        const double d = density[c] * kDensity;
        const double p = pressure[c] * kPressure;
        const double T = std::min(1e-6 * p / (d * kRGas), 5000.);
        const double T1 = kBoltzmann * kPi * T;
        const double T2 = T1 * T1;
        const double T4 = T2 * T2;
        const double Ie = T4 * 2 / (15 * kHPlank * kHPlank * kHPlank * kCLight * kCLight);
        const double betta = d * (kSigmaThomson / kMHydrogen);
        alpha[c] = betta;
        beta[c] = betta;
        Q[c] = betta * Ie;
    }
    *md = rts_medium{};
    md->mode = RTS_MEDIUM_SCATTERING;
    md->s_scale = kDist;
    md->i_scale = kRadiation;
    return RTS_OK;
}

