// standin.hpp -- minimal stand-ins for the types and macros that the
// reference's CPU scattering integral and moment functions use, so that those
// functions can be compiled from the reference's own source text in the
// development container (the reference's headers pull in Eigen, MPI and
// Windows-only headers that are not available).  TEST INFRASTRUCTURE ONLY:
// used by oracle/build_ref.sh; never part of the product.
//
// Stands in for:
//   Type, base ................ global_def.h:23,33 (double, 4 faces)
//   Vector3 (Eigen::Vector3d) . global_def.h:25 -- only dot(), [], +=, /=,
//                               scalar*vector and Zero() are used.  dot() sums
//                               x, y, z left to right.
//   direction_s, grid_directions_t  global_def.h:79-90
//   Matrix3 (Eigen::Matrix3d) . (h,k), Zero(), +=, /= scalar, matrix*vector
//                               (row h: sum over k = 0,1,2 left to right)
//   geo_face_t, face_t, geo_cell_t, illum_value_t, elem_t
//                               solve_module/solve_global_struct.h:86-151
//                               (only the members the divergence code reads)
//   grid_t .................... solve_module/solve_global_struct.h:153-230
//                               (only size, Illum, scattering, cells, faces)
//   MPI_GET_INF ............... global_def.h:157-161 (single process)
#pragma once
#include <cstdint>
#include <cstdio>
#include <vector>
using namespace std;

typedef double Type;
#define base 4

struct Vector3 {
    double v[3];
    Vector3() { v[0] = v[1] = v[2] = 0.0; }
    Vector3(double a, double b, double c) { v[0] = a; v[1] = b; v[2] = c; }
    static Vector3 Zero() { return Vector3(); }
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
    double dot(const Vector3& o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
    Vector3& operator+=(const Vector3& o) { v[0] += o.v[0]; v[1] += o.v[1]; v[2] += o.v[2]; return *this; }
    Vector3& operator/=(double s) { v[0] /= s; v[1] /= s; v[2] /= s; return *this; }
};
inline Vector3 operator*(double s, const Vector3& a) { return Vector3(s * a.v[0], s * a.v[1], s * a.v[2]); }
inline Vector3 operator*(const Vector3& a, double s) { return Vector3(a.v[0] * s, a.v[1] * s, a.v[2] * s); }
inline Vector3 operator-(const Vector3& a) { return Vector3(-a.v[0], -a.v[1], -a.v[2]); }

struct Matrix3 {
    double m[3][3];
    Matrix3() { for (int h = 0; h < 3; ++h) for (int k = 0; k < 3; ++k) m[h][k] = 0.0; }
    static Matrix3 Zero() { return Matrix3(); }
    double& operator()(int h, int k) { return m[h][k]; }
    double operator()(int h, int k) const { return m[h][k]; }
    Matrix3& operator+=(const Matrix3& o) { for (int h = 0; h < 3; ++h) for (int k = 0; k < 3; ++k) m[h][k] += o.m[h][k]; return *this; }
    Matrix3& operator/=(double s) { for (int h = 0; h < 3; ++h) for (int k = 0; k < 3; ++k) m[h][k] /= s; return *this; }
};
inline Vector3 operator*(const Matrix3& a, const Vector3& x)
{
    Vector3 r;
    for (int h = 0; h < 3; ++h) r.v[h] = a.m[h][0] * x.v[0] + a.m[h][1] * x.v[1] + a.m[h][2] * x.v[2];
    return r;
}

struct direction_s { Vector3 dir; Type area; };
struct grid_directions_t { int size; std::vector<direction_s> directions; Type full_area; };
struct geo_face_t { Vector3 n; Type S; };
struct face_t { geo_face_t geo; };
struct geo_cell_t { int id_faces[base]; Type V; bool sign_n[base]; };
struct illum_value_t {
    std::vector<Type> illum;  // [dir][face] of one cell
    Type energy;
    Vector3 stream;
    Matrix3 impuls;
    Type div_stream;
    Vector3 div_impuls;
};
struct elem_t { illum_value_t illum_val; geo_cell_t geo; };
struct grid_t {
    int size;
    Type* Illum;
    Type* scattering;
    std::vector<elem_t> cells;
    std::vector<face_t> faces;
};

#define MPI_GET_INF(np, myid) { np = 1; myid = 0; }

static std::vector<int> send_count;
static std::vector<int> disp;
