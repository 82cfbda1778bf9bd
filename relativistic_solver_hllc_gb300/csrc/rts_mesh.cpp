// rts_mesh.cpp -- host-side geometry of the transport sweep: the synthetic
// cube mesh and the interpolation nodes of every face.
//
// The reference reads its tetrahedral mesh from VTK and precomputes the
// per-face nodes in make_illum_struct; this file builds the same arrays for
// a generated mesh.  Reference paths are relative to solver_hllc_illum_cuda/.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "rts_internal.h"

namespace {

// vertices of face f in VTK's tetra face order, and the vertex off face f
constexpr int kFaceVerts[4][3] = {{0, 1, 3}, {1, 2, 3}, {2, 0, 3}, {0, 2, 1}};
constexpr int kOffFace[4] = {2, 0, 1, 3};

// Outward unit normal of face f, computed as NormalAndSquareFace3D
// (utils/grid_geometry/geometry_data.cpp:141-193): the cross product of the
// face's edges P1-P0 and P2-P0, normalised, turned away from the fourth vertex.
void face_normal(const double* v, int f, double* n)
{
    const double* P0 = v + 3 * kFaceVerts[f][0];
    const double* P1 = v + 3 * kFaceVerts[f][1];
    const double* P2 = v + 3 * kFaceVerts[f][2];
    const double* P3 = v + 3 * kOffFace[f];
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

// The fixed turn of a tilted cube about its centre: Rz(0.1) Ry(0.2) Rx(0.3).
void tilt_point(double* x)
{
    const double a = 0.3, b = 0.2, g = 0.1;
    const double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cg = cos(g), sg = sin(g);
    const double p0 = x[0] - 0.5, p1 = x[1] - 0.5, p2 = x[2] - 0.5;
    const double q1 = ca * p1 - sa * p2, q2 = sa * p1 + ca * p2;
    const double r0 = cb * p0 + sb * q2, r2 = -sb * p0 + cb * q2;
    x[0] = cg * r0 - sg * q1 + 0.5;
    x[1] = sg * r0 + cg * q1 + 0.5;
    x[2] = r2 + 0.5;
}

}  // namespace

void rts_face_normals_host(int64_t N, const double* vert, double* normals)
{
    for (int64_t c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f) face_normal(vert + 12 * c, f, normals + 12 * c + 3 * f);
}

// MakeArrayX (make_illum_struct/struct_short_characteristics_logic_function.cpp:
// 10-73): the 3 nodes of face f sit at the local coordinates of the rows of
// straight_face ({1/6,1/6}, {2/3,1/6}, {1/6,2/3}) on the coordinate plane the
// face lies in, or for face 3 at the rows of inclined_face carried from the
// inclined plane by inverse_transform_matrix and start_point_plane_coord
// (struct_short_characteristics_calculations.cpp:102-128,146-183); local coordinates
// xi map to sum_j V_j xi_j + V_3 (1 - xi_0 - xi_1 - xi_2) (FromLocalToGlobalTetra).
void rts_sweep_nodes_host(int64_t N, const double* vert, double* nodes)
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
                switch (f) {
                case 0: xi[0] = straight[m][0], xi[1] = straight[m][1], xi[2] = 0; break;
                case 1: xi[0] = 0, xi[1] = straight[m][0], xi[2] = straight[m][1]; break;
                case 2: xi[0] = straight[m][0], xi[1] = 0, xi[2] = straight[m][1]; break;
                default: {
                    const double p[3] = {inclined[m][0], inclined[m][1], 0};
                    for (int i = 0; i < 3; ++i)
                        xi[i] = inv_t[i][0] * p[0] + inv_t[i][1] * p[1] + inv_t[i][2] * p[2] + start[i];
                }
                }
                const double eta4 = 1 - xi[0] - xi[1] - xi[2];
                double* x = nodes + 36 * c + 9 * f + 3 * m;
                for (int i = 0; i < 3; ++i) {
                    double g = 0;
                    for (int j = 0; j < 3; ++j) g += v[3 * j + i] * xi[j];
                    g += v[9 + i] * eta4;
                    x[i] = g;
                }
            }
    }
}

extern "C" int rts_mesh_cube(int n, int bound_rule, int tilt, double* vert, int32_t* pairs, double* normals)
{
    static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    if (n < 1 || n > 127 || !vert || !pairs || !normals || bound_rule < 0 || bound_rule > 1)
        return RTS_ERR_INVALID_ARGUMENT;
    const int64_t N = 6 * (int64_t)n * n * n, np1 = n + 1;
    std::vector<int64_t> pid(4 * N);
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const int64_t h = ((int64_t)k * n + j) * n + i;
                for (int t = 0; t < 6; ++t) {
                    const int64_t c = 6 * h + t;
                    int p[3] = {i, j, k};
                    for (int q = 0; q < 4; ++q) {
                        if (q == 1 || q == 2) p[perm[t][q - 1]] += 1;
                        if (q == 3) p[0] = i + 1, p[1] = j + 1, p[2] = k + 1;
                        double* v = vert + 12 * c + 3 * q;
                        for (int a = 0; a < 3; ++a) v[a] = (double)p[a] / (double)n;
                        pid[4 * c + q] = ((int64_t)p[2] * np1 + p[1]) * np1 + p[0];
                    }
                }
            }
    rts_face_normals_host(N, vert, normals);
    // faces are matched by their sorted vertex ids (21 bits each)
    std::vector<std::pair<uint64_t, int64_t>> keys(4 * N);
    for (int64_t c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f) {
            int64_t a = pid[4 * c + kFaceVerts[f][0]], b = pid[4 * c + kFaceVerts[f][1]], d = pid[4 * c + kFaceVerts[f][2]];
            if (a > b) std::swap(a, b);
            if (b > d) std::swap(b, d);
            if (a > b) std::swap(a, b);
            keys[4 * c + f] = {((uint64_t)a << 42) | ((uint64_t)b << 21) | (uint64_t)d, 4 * c + f};
        }
    std::sort(keys.begin(), keys.end());
    for (size_t i = 0; i < keys.size();) {
        if (i + 1 < keys.size() && keys[i + 1].first == keys[i].first) {
            pairs[keys[i].second] = (int32_t)keys[i + 1].second;
            pairs[keys[i + 1].second] = (int32_t)keys[i].second;
            i += 2;
            continue;
        }
        const int64_t id = keys[i].second;
        const double* nn = normals + 3 * id;
        int code = RTS_BOUND_FREE;
        if (bound_rule == 1) {
            const double dm = sqrt((nn[0] + 1) * (nn[0] + 1) + nn[1] * nn[1] + nn[2] * nn[2]);
            const double dp = sqrt((nn[0] - 1) * (nn[0] - 1) + nn[1] * nn[1] + nn[2] * nn[2]);
            code = dm < 1e-7 ? RTS_BOUND_OUTSOURCE : dp < 1e-7 ? RTS_BOUND_FREE : RTS_BOUND_LOCK;
        }
        pairs[id] = code;
        i += 1;
    }
    if (tilt) {
        for (int64_t i = 0; i < 4 * N; ++i) tilt_point(vert + 3 * i);
        rts_face_normals_host(N, vert, normals);
    }
    return RTS_OK;
}
