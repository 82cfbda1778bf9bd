/*
 * sweep_oracle.c -- CPU oracle of the transport sweep that produces Illum.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file.  tests/ use it as the checker of the device sweep, and
 * bench.py's CPU-baseline leg of the sweep times it.
 *
 * What it restates (reference paths are relative to solver_hllc_illum_cuda/):
 *   orc_face_normals ... outward unit face normals, NormalAndSquareFace3D
 *                        (utils/grid_geometry/geometry_data.cpp:141-193): the
 *                        cross product of the face's first two edges,
 *                        normalised, pointing away from the fourth vertex
 *   orc_sweep_nodes .... MakeArrayX (make_illum_struct/
 *                        struct_short_characteristics_logic_function.cpp:10-73)
 *                        with FromLocalToGlobalTetra, FromPlaneToTetra and the
 *                        BaseTetra_t constants
 *                        (struct_short_characteristics_calculations.cpp:102-128,146-183)
 *   face states ........ GetInAndOutFaces (utils/grid_geometry/geometry_solve.cpp:212-227)
 *   orc_sweep_graph .... build_graph's cell order: FindNumberOfAllInnerFaceAndKnew,
 *                        FindCurCell, NewStep (build_graph/build_graph_calculation.cpp:
 *                        347-391,482-510) driven as in build_graph/build_graph_main.cpp:165-300
 *   orc_sweep_x0 ....... GetNodes / CalculateNodeValue (logic_function.cpp:222-297)
 *                        with IntersectionWithPlane, InTriangle, SetBasis,
 *                        Make2dPoint (geometry_solve.cpp:8-56,109-159)
 *   orc_sweep_dir ...... one direction of the sweep in MPI_CalculateIllumAsync
 *                        (solve_module/illum/Illum_async.cpp:726-784) with
 *                        CalculateIllumeOnInnerFace (:172-199), GetCurIllum
 *                        (:259-470, as a parametrised medium), ReCalcIllum
 *                        (:472-510) and BoundaryConditions
 *                        (solve_module/illum/illum_utils.cpp:407-474)
 *   orc_cube_mesh ...... the synthetic mesh: the unit cube cut into n^3 hexahedra,
 *                        each cut into 6 tetrahedra around its main diagonal,
 *                        with face pairs and boundary codes (the reference reads
 *                        a VTK mesh instead; the boundary rules are its `Cube`
 *                        and `Cone` variants of SetTypeOfBound,
 *                        utils/grid_geometry/geometry_data.cpp:472-520)
 *
 * Operation order follows the reference where it fixes the result: the node
 * positions, the plane intersection, the 2-D in-triangle test, the 3-node
 * means and GetCurIllum's expression.  The medium of GetCurIllum is
 * parametrised: mode 0 is the scattering form of classes 0, 1, 3, 10 and 11
 * with per-cell alpha, beta, Q, a distance scale (DIST for class 11) and an
 * intensity scale (RADIATION for class 11), and an optional ball where other
 * coefficients hold (class 0); mode 1 is the pure absorption form of class 2.
 *
 * Parity pin: oracle/build_ref.sh compiles the reference's own GetCurIllum,
 * ReCalcIllum, BoundaryConditions, CalculateIllumeOnInnerFace, the sweep loop
 * body and the geometry functions from the reference source text (development
 * container only); tests/golden/make_golden.py ran them on small cube meshes
 * and tests/test_sweep_golden.py checks this restatement against the stored
 * outputs (bit for bit).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SW_EPS 1e-10 /* `eps` in global_value.h:13 */

/* vertices of face f of a tetrahedron, in VTK's face order (the order the
 * reference's grid.bin and normals come in) */
static const int SW_FV[4][3] = {{0, 1, 3}, {1, 2, 3}, {2, 0, 3}, {0, 2, 1}};
/* the vertex not on face f */
static const int SW_OPP[4] = {2, 0, 1, 3};

/* boundary codes of eBoundaryTypes (global_def.h:45-51) */
enum { SW_FREE = -1, SW_LOCK = -2, SW_OUTSOURCE = -3, SW_INNER = -4 };

/* ------------------------------------------------------------------ */
/* synthetic mesh                                                       */
/* ------------------------------------------------------------------ */

int64_t orc_cube_cells(int n) { return 6 * (int64_t)n * n * n; }

typedef struct {
    uint64_t key;
    int64_t face;
} sw_facekey;

static int sw_cmp_key(const void* a, const void* b)
{
    const sw_facekey* x = (const sw_facekey*)a;
    const sw_facekey* y = (const sw_facekey*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->face < y->face ? -1 : (x->face > y->face);
}

/* outward unit normal of face f of the tetrahedron v[4][3] */
static void sw_face_normal(const double* v, int f, double* n)
{
    const double* P0 = v + 3 * SW_FV[f][0];
    const double* P1 = v + 3 * SW_FV[f][1];
    const double* P2 = v + 3 * SW_FV[f][2];
    const double* P3 = v + 3 * SW_OPP[f];
    double a[3], b[3];
    for (int i = 0; i < 3; ++i) {
        a[i] = P1[i] - P0[i];
        b[i] = P2[i] - P0[i];
    }
    n[0] = a[1] * b[2] - a[2] * b[1];
    n[1] = -a[0] * b[2] + a[2] * b[0];
    n[2] = a[0] * b[1] - a[1] * b[0];
    const double z = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int i = 0; i < 3; ++i) n[i] /= z;
    const double side = n[0] * (P3[0] - P0[0]) + n[1] * (P3[1] - P0[1]) + n[2] * (P3[2] - P0[2]);
    if (side > 0)
        for (int i = 0; i < 3; ++i) n[i] = -n[i];
}

void orc_face_normals(int64_t N, const double* vert, double* normals)
{
    for (int64_t c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f) sw_face_normal(vert + 12 * c, f, normals + 12 * c + 3 * f);
}

/* Unit cube, n^3 hexahedra (i fastest), each cut into 6 tetrahedra around
 * the diagonal from its corner (0,0,0) to (1,1,1): tetrahedron t follows the
 * axis permutation perm[t] from the first corner to the last.  vert
 * [N][4][3], pairs [N][4] (cell*4 + face of the neighbour, or a boundary
 * code), normals [N][4][3] (outward, unit).  bound_rule 0: every boundary
 * face FreeBound; 1: the x = 0 faces OutSource, the x = 1 faces FreeBound,
 * the rest LockBound.  tilt != 0 turns the cube about its centre by the fixed
 * rotation of sw_tilt (the boundary codes keep the faces of the unturned
 * cube): with an axis-aligned cube, directions parallel to a face (the first
 * spherical-Fibonacci direction has y = 0) send characteristics along
 * edges, where no in-face contains the back-traced point.  Returns 0, or -1
 * for n outside [1, 127]. */
static void sw_tilt(double* x)
{
    const double a = 0.3, b = 0.2, g = 0.1; /* rotation Rz(g) Ry(b) Rx(a) */
    const double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cg = cos(g), sg = sin(g);
    const double p0 = x[0] - 0.5, p1 = x[1] - 0.5, p2 = x[2] - 0.5;
    const double q1 = ca * p1 - sa * p2, q2 = sa * p1 + ca * p2;  /* Rx */
    const double r0 = cb * p0 + sb * q2, r2 = -sb * p0 + cb * q2; /* Ry */
    x[0] = cg * r0 - sg * q1 + 0.5;                                /* Rz */
    x[1] = sg * r0 + cg * q1 + 0.5;
    x[2] = r2 + 0.5;
}

int orc_cube_mesh(int n, int bound_rule, int tilt, double* vert, int32_t* pairs, double* normals)
{
    static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    if (n < 1 || n > 127) return -1;
    const int64_t N = orc_cube_cells(n);
    const int64_t np1 = n + 1;
    int64_t* pid = (int64_t*)malloc(sizeof(int64_t) * 4 * N);
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const int64_t h = ((int64_t)k * n + j) * n + i;
                for (int t = 0; t < 6; ++t) {
                    const int64_t c = 6 * h + t;
                    int p[3] = {i, j, k};
                    for (int q = 0; q < 4; ++q) {
                        if (q > 0 && q < 3) p[perm[t][q - 1]] += 1;
                        if (q == 3) p[0] = i + 1, p[1] = j + 1, p[2] = k + 1;
                        double* v = vert + 12 * c + 3 * q;
                        v[0] = (double)p[0] / (double)n;
                        v[1] = (double)p[1] / (double)n;
                        v[2] = (double)p[2] / (double)n;
                        pid[4 * c + q] = ((int64_t)p[2] * np1 + p[1]) * np1 + p[0];
                    }
                }
            }
    orc_face_normals(N, vert, normals);
    sw_facekey* keys = (sw_facekey*)malloc(sizeof(sw_facekey) * 4 * N);
    for (int64_t c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f) {
            int64_t a = pid[4 * c + SW_FV[f][0]], b = pid[4 * c + SW_FV[f][1]], d = pid[4 * c + SW_FV[f][2]], t;
            if (a > b) t = a, a = b, b = t;
            if (b > d) t = b, b = d, d = t;
            if (a > b) t = a, a = b, b = t;
            keys[4 * c + f].key = ((uint64_t)a << 42) | ((uint64_t)b << 21) | (uint64_t)d;
            keys[4 * c + f].face = 4 * c + f;
        }
    qsort(keys, (size_t)(4 * N), sizeof(sw_facekey), sw_cmp_key);
    for (int64_t i = 0; i < 4 * N;) {
        if (i + 1 < 4 * N && keys[i + 1].key == keys[i].key) {
            pairs[keys[i].face] = (int32_t)keys[i + 1].face;
            pairs[keys[i + 1].face] = (int32_t)keys[i].face;
            i += 2;
            continue;
        }
        const int64_t id = keys[i].face;
        const double* nn = normals + 3 * id;
        int code = SW_FREE;
        if (bound_rule == 1) {
            const double dm = sqrt((nn[0] + 1) * (nn[0] + 1) + nn[1] * nn[1] + nn[2] * nn[2]);
            const double dp = sqrt((nn[0] - 1) * (nn[0] - 1) + nn[1] * nn[1] + nn[2] * nn[2]);
            code = dm < 1e-7 ? SW_OUTSOURCE : dp < 1e-7 ? SW_FREE : SW_LOCK;
        }
        pairs[id] = code;
        i += 1;
    }
    free(keys);
    free(pid);
    if (tilt) {
        for (int64_t i = 0; i < 4 * N; ++i) sw_tilt(vert + 3 * i);
        orc_face_normals(N, vert, normals);
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* MakeArrayX: the 3 nodes of every face                                */
/* ------------------------------------------------------------------ */

/* local (barycentric-like) coordinates xi[3] -> global point, as
 * FromLocalToGlobalTetra: sum_j V_j xi_j + V_3 (1 - xi_0 - xi_1 - xi_2) */
static void sw_local_to_global(const double* v, const double* xi, double* x)
{
    const double eta4 = 1 - xi[0] - xi[1] - xi[2];
    for (int i = 0; i < 3; ++i) {
        double g = 0;
        for (int j = 0; j < 3; ++j) g += v[3 * j + i] * xi[j];
        g += v[9 + i] * eta4;
        x[i] = g;
    }
}

/* nodes [N][4][3][3]: node m of face f of cell c */
void orc_sweep_nodes(int64_t N, const double* vert, double* nodes)
{
    const double straight[3][2] = {{1. / 6, 1. / 6}, {2. / 3, 1. / 6}, {1. / 6, 2. / 3}};
    const double inclined[3][2] = {
        {0, sqrt(2. / 3)}, {sqrt(2) / 4, 1. / (2 * sqrt(6))}, {-sqrt(2) / 4, 1. / (2 * sqrt(6))}};
    const double inv_t[3][3] = {{-1. / sqrt(2), -1. / sqrt(6), 1. / sqrt(3)},
                                {1. / sqrt(2), -1. / sqrt(6), 1. / sqrt(3)},
                                {0, sqrt(2. / 3), 1. / sqrt(3)}};
    const double start[3] = {0.5, 0.5, 0};
    for (int64_t c = 0; c < N; ++c) {
        const double* v = vert + 12 * c;
        for (int f = 0; f < 4; ++f)
            for (int m = 0; m < 3; ++m) {
                double xi[3];
                if (f == 1) {
                    xi[0] = 0, xi[1] = straight[m][0], xi[2] = straight[m][1];
                } else if (f == 2) {
                    xi[0] = straight[m][0], xi[1] = 0, xi[2] = straight[m][1];
                } else if (f == 0) {
                    xi[0] = straight[m][0], xi[1] = straight[m][1], xi[2] = 0;
                } else {
                    const double p[3] = {inclined[m][0], inclined[m][1], 0};
                    for (int i = 0; i < 3; ++i) xi[i] = inv_t[i][0] * p[0] + inv_t[i][1] * p[1] + inv_t[i][2] * p[2] + start[i];
                }
                sw_local_to_global(v, xi, nodes + 36 * c + 9 * f + 3 * m);
            }
    }
}

/* ------------------------------------------------------------------ */
/* face states, cell order                                              */
/* ------------------------------------------------------------------ */

/* bit f set: face f is an in-face (n_f . dir < -eps), GetInAndOutFaces */
static int sw_state(const double* nrm, const double* dir)
{
    int st = 0;
    for (int f = 0; f < 4; ++f) {
        const double* n = nrm + 3 * f;
        if (n[0] * dir[0] + n[1] * dir[1] + n[2] * dir[2] < -SW_EPS) st |= 1 << f;
    }
    return st;
}

void orc_face_states(int64_t N, const double* normals, const double* dir, int32_t* states)
{
    for (int64_t c = 0; c < N; ++c) states[c] = sw_state(normals + 12 * c, dir);
}

static int sw_cmp_i32(const void* a, const void* b)
{
    const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

/* build_graph's cell order for one direction: cells whose in-faces all have
 * known values, step by step; each step's cells in ascending id (the
 * reference keeps them in a std::set).  order [N]; level_off [N+1] receives
 * the first position of every step and the end; returns the number of steps,
 * or -1 when the graph cannot be completed (a dependency cycle). */
int64_t orc_sweep_graph(int64_t N, const int32_t* pairs, const int32_t* states, int32_t* order, int64_t* level_off)
{
    int32_t* count_in = (int32_t*)calloc((size_t)N, sizeof(int32_t));
    int32_t* knew = (int32_t*)calloc((size_t)N, sizeof(int32_t));
    char* in_next = (char*)calloc((size_t)N, 1);
    int32_t* next = (int32_t*)malloc(sizeof(int32_t) * (size_t)(N > 0 ? N : 1));
    int64_t nnext = 0, done = 0, levels = 0;
    for (int64_t c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f)
            if ((states[c] >> f) & 1) {
                count_in[c]++;
                if (pairs[4 * c + f] < 0) {
                    knew[c]++;
                    if (!in_next[c]) in_next[c] = 1, next[nnext++] = (int32_t)c;
                }
            }
    while (nnext > 0) {
        qsort(next, (size_t)nnext, sizeof(int32_t), sw_cmp_i32);
        const int64_t lv0 = done;
        for (int64_t i = 0; i < nnext; ++i) {
            in_next[next[i]] = 0;
            if (count_in[next[i]] == knew[next[i]]) order[done++] = next[i];
        }
        if (done == lv0) break;
        level_off[levels++] = lv0;
        nnext = 0;
        for (int64_t i = lv0; i < done; ++i) {
            const int64_t c = order[i];
            for (int f = 0; f < 4; ++f) {
                int32_t nb = pairs[4 * c + f];
                if (nb < 0) continue;
                nb /= 4;
                if (count_in[nb] > knew[nb]) {
                    knew[nb]++;
                    if (!in_next[nb]) in_next[nb] = 1, next[nnext++] = nb;
                }
            }
        }
    }
    level_off[levels] = done;
    free(count_in);
    free(knew);
    free(in_next);
    free(next);
    return done == N ? levels : -1;
}

/* ------------------------------------------------------------------ */
/* short characteristics: the in-face and distance of every out-face node */
/* ------------------------------------------------------------------ */

/* IntersectionWithPlane: the line start + t dir meets the plane of the face
 * (A, B, C) */
static void sw_intersect(const double* A, const double* B, const double* C, const double* x, const double* dir,
                         double* res)
{
    const double a = A[1] * (B[2] - C[2]) + B[1] * (C[2] - A[2]) + C[1] * (A[2] - B[2]);
    const double b = A[0] * (C[2] - B[2]) + B[0] * (A[2] - C[2]) + C[0] * (B[2] - A[2]);
    const double c = A[0] * (B[1] - C[1]) + B[0] * (C[1] - A[1]) + C[0] * (A[1] - B[1]);
    const double d = A[0] * (C[1] * B[2] - B[1] * C[2]) + B[0] * (A[1] * C[2] - C[1] * A[2]) +
                     C[0] * (B[1] * A[2] - A[1] * B[2]);
    const double t = -(a * x[0] + b * x[1] + c * x[2] + d) / (a * dir[0] + b * dir[1] + c * dir[2]);
    for (int i = 0; i < 3; ++i) res[i] = dir[i] * t + x[i];
}

/* InTriangle: X in the triangle (A, B, C) of the plane with normal n, tested
 * in a 2-D frame of that plane built as SetBasis / Make2dPoint */
static int sw_in_triangle(const double* A, const double* B, const double* C, const double* n, const double* X)
{
    double v1[3], v2[3];
    if (fabs(n[1]) < 1e-20) {
        v1[0] = 0, v1[1] = 1, v1[2] = 0;
    } else {
        v1[0] = 1, v1[2] = 0;
        v1[1] = -(n[0] * v1[0] + n[2] * v1[2]) / n[1];
    }
    if (n[1] < 0)
        for (int i = 0; i < 3; ++i) v1[i] *= -1;
    v2[0] = -(n[1] * v1[2] - n[2] * v1[1]);
    v2[1] = -(n[2] * v1[0] - n[0] * v1[2]);
    v2[2] = -(n[0] * v1[1] - n[1] * v1[0]);
    const double z1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    const double z2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
    for (int i = 0; i < 3; ++i) v1[i] /= z1, v2[i] /= z2;
    const double* P[4] = {A, B, C, X};
    double q[4][2];
    for (int p = 0; p < 4; ++p) {
        double u = 0, w = 0;
        for (int k = 0; k < 3; ++k) {
            u += (P[p][k] - A[k]) * v1[k];
            w += (P[p][k] - A[k]) * v2[k];
        }
        q[p][0] = u, q[p][1] = w;
    }
    const double* a = q[0];
    const double* b = q[1];
    const double* c = q[2];
    const double* x = q[3];
    const double r1 = (a[0] - x[0]) * (b[1] - a[1]) - (b[0] - a[0]) * (a[1] - x[1]);
    const double r2 = (b[0] - x[0]) * (c[1] - b[1]) - (c[0] - b[0]) * (b[1] - x[1]);
    const double r3 = (c[0] - x[0]) * (a[1] - c[1]) - (a[0] - c[0]) * (c[1] - x[1]);
    if (r1 < 0 && r2 < 0 && r3 < 0) return 1;
    if (r1 > 0 && r2 > 0 && r3 > 0) return 1;
    return 0;
}

/* The x0 records of one direction in the reference's LocX0 order: for every
 * cell in `order`, every out-face in ascending order, its 3 nodes.  s [nx]
 * distances to the in-face hit going back along the direction, face [nx] the
 * in-face.  Returns the record count, or -(1 + position) of the first node
 * whose in-face was not found. */
int64_t orc_sweep_x0(int64_t N, const double* vert, const double* normals, const double* nodes, const int32_t* order,
                     const int32_t* states, const double* dir, double* s, int8_t* face)
{
    int64_t pos = 0;
    for (int64_t h = 0; h < N; ++h) {
        const int64_t c = order[h];
        const double* v = vert + 12 * c;
        for (int f = 0; f < 4; ++f) {
            if ((states[c] >> f) & 1) continue;
            for (int m = 0; m < 3; ++m) {
                const double* x = nodes + 36 * c + 9 * f + 3 * m;
                int found = -1;
                for (int g = 0; g < 4 && found < 0; ++g) {
                    if (!((states[c] >> g) & 1)) continue;
                    const double* A = v + 3 * SW_FV[g][0];
                    const double* B = v + 3 * SW_FV[g][1];
                    const double* C = v + 3 * SW_FV[g][2];
                    double x0[3];
                    sw_intersect(A, B, C, x, dir, x0);
                    if (sw_in_triangle(A, B, C, normals + 12 * c + 3 * g, x0)) {
                        const double d0 = x[0] - x0[0], d1 = x[1] - x0[1], d2 = x[2] - x0[2];
                        s[pos] = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                        face[pos] = (int8_t)g;
                        found = g;
                    }
                }
                if (found < 0) return -(1 + pos);
                ++pos;
            }
        }
    }
    return pos;
}

/* ------------------------------------------------------------------ */
/* the sweep                                                            */
/* ------------------------------------------------------------------ */

typedef struct {
    int mode;                 /* 0 scattering form, 1 absorption form */
    int reserved;
    double s_scale, i_scale;  /* distance and intensity units */
    double ball[3], radius;   /* radius > 0: inside the ball the ball_* coefficients hold */
    double ball_alpha, ball_beta, ball_q;
} orc_medium;

/* GetCurIllum with the medium's coefficients at point x of cell c */
static double sw_cur_illum(const orc_medium* md, double alpha, double betta, double Q, const double* x, double s,
                           double I_0, double int_scattering)
{
    if (md->radius > 0) {
        const double d0 = x[0] - md->ball[0], d1 = x[1] - md->ball[1], d2 = x[2] - md->ball[2];
        if (sqrt(d0 * d0 + d1 * d1 + d2 * d2) < md->radius) alpha = md->ball_alpha, betta = md->ball_beta, Q = md->ball_q;
    }
    double I;
    if (md->mode == 1) {
        const double ss = s * md->s_scale;
        if (alpha > 1e-15)
            I = I_0 * exp(-alpha * ss) + Q * (1 - exp(-alpha * ss)) / alpha;
        else
            I = I_0 * (1 - alpha * ss) + Q * ss;
        if (I < 0) return 0;
        return I;
    }
    const double S = int_scattering * md->i_scale;
    const double ss = s * md->s_scale;
    const double I0 = I_0 * md->i_scale;
    const double k = alpha + betta;
    if (k > 1e-10)
        I = (exp(-k * ss) * (I0 * k + (exp(k * ss) - 1) * (Q + S * betta))) / k;
    else
        I = (1 - ss * k) * (I0 + ss * (Q + S * betta));
    if (I < 0) return 0;
    return I / md->i_scale;
}

/* Class 11 of GetCurIllum (Illum_async.cpp:419-447) as a medium: per cell
 * alpha = beta = d (sigma_thomson / m_hydrogen), Q = alpha Ie(T) from the gas
 * density and pressure in code units, with the reference's units and
 * constants (global_value.h:32-52, the macros expanded as written there);
 * the medium gets s_scale = DIST, i_scale = RADIATION. */
void orc_medium_gas(int64_t N, const double* density, const double* pressure, double* alpha, double* beta, double* Q,
                    orc_medium* md)
{
    const double PI_ = 3.14159265358979323846, C_LIGHT_ = 299792458.0;
    const double DENSITY_ = (3.34 * 10e-14), VELOCITY_ = (3 * 1e8);
    const double PRESSURE_ = (DENSITY_ * VELOCITY_ * VELOCITY_);
    const double RADIATION_ = (DENSITY_ * VELOCITY_ * VELOCITY_ * VELOCITY_);
    const double R_gas = 8.314, h_plank = 6.62 * 1e-34, k_boltzmann = 1.38 * 1e-23;
    const double sigma_thomson = 6.652 * 1e-29, m_hydrogen = 1.6735575 * 1e-27;
    for (int64_t c = 0; c < N; ++c) {
        const double d = density[c] * DENSITY_;
        const double p = pressure[c] * PRESSURE_;
        double T = 1e-6 * p / (d * R_gas);
        if (T > 5000.) T = 5000.;
        const double T1 = k_boltzmann * PI_ * T;
        const double T2 = T1 * T1;
        const double T4 = T2 * T2;
        const double Ie = T4 * 2 / (15 * h_plank * h_plank * h_plank * C_LIGHT_ * C_LIGHT_);
        const double betta = d * (sigma_thomson / m_hydrogen);
        alpha[c] = betta;
        beta[c] = betta;
        Q[c] = betta * Ie;
    }
    memset(md, 0, sizeof(*md));
    md->mode = 0;
    md->s_scale = 1e6;
    md->i_scale = RADIATION_;
}

/* One direction: cells in `order`, x0 records (s, face) in the same order,
 * S [N] the scattering of this direction, bc [4] the intensities of boundary
 * codes -1..-4, coef [N*4*3] scratch; writes illum [N][4] (face means) and
 * returns ReCalcIllum's norm max |old - new| / new over the faces (-1 when
 * every term is NaN). */
double orc_sweep_dir(int64_t N, const int32_t* pairs, const double* nodes, const int32_t* order, const int32_t* states,
                     const double* s, const int8_t* face, const double* S, const orc_medium* md, const double* alpha,
                     const double* beta, const double* Q, const double* bc, double* illum, double* coef)
{
    int64_t pos = 0;
    static const double origin[3] = {0, 0, 0};
    for (int64_t h = 0; h < N; ++h) {
        const int64_t c = order[h];
        const int64_t fb = 4 * c;
        for (int f = 0; f < 4; ++f) {
            const int32_t out_id = pairs[fb + f];
            if ((states[c] >> f) & 1) {
                if (out_id < 0) {
                    const double I0 = bc[-out_id - 1];
                    double* k = coef + 3 * (fb + f);
                    k[0] = k[1] = k[2] = I0;
                }
                continue;
            }
            double I[3];
            for (int m = 0; m < 3; ++m) {
                const int g = face[pos];
                const double sv = s[pos];
                ++pos;
                const int32_t nb = pairs[fb + g];
                double I_x0;
                if (nb < 0) {
                    I_x0 = bc[-nb - 1];
                    double* k = coef + 3 * (fb + g);
                    k[0] = k[1] = k[2] = I_x0;
                } else {
                    const double* k = coef + 3 * (fb + g);
                    I_x0 = (k[0] + k[1] + k[2]) / 3;
                }
                const double* x = nodes ? nodes + 36 * c + 9 * f + 3 * m : origin;
                I[m] = sw_cur_illum(md, alpha[c], beta[c], Q[c], x, sv, I_x0, S[c]);
            }
            double* k = coef + 3 * (fb + f);
            k[0] = I[0], k[1] = I[1], k[2] = I[2];
            if (out_id >= 0) {
                double* kn = coef + 3 * (int64_t)out_id;
                kn[0] = I[0], kn[1] = I[1], kn[2] = I[2];
            }
        }
    }
    double norm = -1;
    for (int64_t c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f) {
            const double* k = coef + 3 * (4 * c + f);
            const double curI = (k[0] + k[1] + k[2]) / 3;
            const int64_t id = 4 * c + f;
            const double buf = fabs(illum[id] - curI) / curI;
            if (buf > norm) norm = buf;
            illum[id] = curI;
        }
    return norm;
}

/* Every direction d of [0, D): order/states [D][N], records (s, face) of
 * direction d from rec_off[d], S [D][N], illum [D][N][4]; OpenMP over
 * directions (nthreads <= 0: the runtime's default).  Returns the max norm. */
double orc_sweep_all(int64_t N, int64_t D, const int32_t* pairs, const double* nodes, const int32_t* order,
                     const int32_t* states, const int64_t* rec_off, const double* s, const int8_t* face,
                     const double* S, const orc_medium* md, const double* alpha, const double* beta, const double* Q,
                     const double* bc, double* illum, int nthreads)
{
    double norm = -1;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        double* coef = (double*)calloc((size_t)(12 * N), sizeof(double));
        double loc = -1;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int64_t d = 0; d < D; ++d) {
            const double r = orc_sweep_dir(N, pairs, nodes, order + d * N, states + d * N, s + rec_off[d],
                                           face + rec_off[d], S + d * N, md, alpha, beta, Q, bc, illum + 4 * d * N, coef);
            if (r > loc) loc = r;
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        if (loc > norm) norm = loc;
        free(coef);
    }
    (void)nthreads;
    return norm;
}
