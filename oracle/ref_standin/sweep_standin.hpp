// sweep_standin.hpp -- minimal stand-ins for the types, constants and macros
// that the reference's transport sweep, its characteristic geometry
// (make_illum_struct) and its cell ordering (build_graph) use, so that those
// functions can be compiled from the reference's own source text in the
// development container.  TEST INFRASTRUCTURE ONLY: used by
// oracle/build_ref.sh; never part of the product.
//
// Stands in for (reference paths relative to solver_hllc_illum_cuda/):
//   Type, base, ShortId, IntId ....... global_def.h:23,33-37
//   Vector3 / Vector2 / Matrix3 / Matrix4 (Eigen) -- only what the compiled
//   functions use: [], (), data(), dot(), cross(), norm(), normalize(),
//   + - between vectors, scalar products, row(i) read and assignment, the
//   comma initializer, inverse() (3x3, cofactors), matrix * vector with each
//   row summed left to right
//   Normals, Face, FaceCell, cell_local, BasePointTetra  global_def.h:53-108
//   eBoundaryTypes ................... global_def.h:45-51
//   check_bit / set_bit / clear_bit .. global_def.h:194-196
//   eps, physical constants, units .. global_value.h:8-52 (values as there)
//   flux_t, solve_mode_t, grid_t ..... solve_module/solve_global_struct.h
//                                      (only the members the code reads)
//   BaseTetra_t ...................... make_illum_struct/
//                                      struct_short_characteristics_global_structure.h:9-28
//   RETURN_ERR / EXIT_ERR / D_LD ..... report through ref_failed instead of
//                                      printing and exiting
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <bitset>
#include <iostream>
#include <list>
#include <map>
#include <set>
#include <vector>
using namespace std;

typedef double Type;
typedef int IntId;
typedef uint8_t ShortId;
typedef int State;
#define base 4
#define NUMBER_OF_MEASUREMENTS 3

static int ref_failed = 0;
#define RETURN_ERR(str) { ref_failed = 1; return 1; }
#define RETURN_ERRS(str, val) { ref_failed = 1; return 1; }
#define EXIT_ERR(str) { ref_failed = 1; return 1; }
#define EXIT_ERRS(str, val) { ref_failed = 1; return Vector2(0, 0); }
#define D_LD { ref_failed = 2; }
#define WRITE_LOG(str) {}

struct Vector3 {
    double v[3];
    Vector3() { v[0] = v[1] = v[2] = 0.0; }
    Vector3(double a, double b, double c) { v[0] = a; v[1] = b; v[2] = c; }
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
    double& operator()(int i) { return v[i]; }
    double operator()(int i) const { return v[i]; }
    double* data() { return v; }
    const double* data() const { return v; }
    double dot(const Vector3& o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
    double squaredNorm() const { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
    double norm() const { return std::sqrt(squaredNorm()); }
    void normalize()
    {
        const double z = squaredNorm();
        if (z > 0) {
            const double n = std::sqrt(z);
            v[0] /= n; v[1] /= n; v[2] /= n;
        }
    }
    struct Comma {
        Vector3& V;
        int i;
        Comma& operator,(double x) { V.v[i++] = x; return *this; }
    };
    Comma operator<<(double x) { v[0] = x; return Comma{*this, 1}; }
    Vector3 cross(const Vector3& o) const
    {
        return Vector3(v[1] * o.v[2] - v[2] * o.v[1], v[2] * o.v[0] - v[0] * o.v[2], v[0] * o.v[1] - v[1] * o.v[0]);
    }
};
inline Vector3 operator+(const Vector3& a, const Vector3& b) { return Vector3(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
inline Vector3 operator-(const Vector3& a, const Vector3& b) { return Vector3(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
inline Vector3 operator*(double s, const Vector3& a) { return Vector3(s * a.v[0], s * a.v[1], s * a.v[2]); }
inline Vector3 operator*(const Vector3& a, double s) { return Vector3(a.v[0] * s, a.v[1] * s, a.v[2] * s); }

struct Vector2 {
    double v[2];
    Vector2() { v[0] = v[1] = 0.0; }
    Vector2(double a, double b) { v[0] = a; v[1] = b; }
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
};

struct Matrix3 {
    double m[3][3];
    struct Row {
        double* p;
        double operator[](int k) const { return p[k]; }
        Row& operator=(const Vector3& x) { p[0] = x.v[0]; p[1] = x.v[1]; p[2] = x.v[2]; return *this; }
    };
    struct CRow {
        const double* p;
        double operator[](int k) const { return p[k]; }
    };
    struct Comma {
        Matrix3& M;
        int i;
        Comma& operator,(double x) { M.m[i / 3][i % 3] = x; ++i; return *this; }
    };
    Matrix3() { for (int h = 0; h < 3; ++h) for (int k = 0; k < 3; ++k) m[h][k] = 0.0; }
    double& operator()(int h, int k) { return m[h][k]; }
    double operator()(int h, int k) const { return m[h][k]; }
    Row row(int h) { return Row{m[h]}; }
    CRow row(int h) const { return CRow{m[h]}; }
    Comma operator<<(double x) { m[0][0] = x; return Comma{*this, 1}; }
    Matrix3 inverse() const
    {
        const double a = m[0][0], b = m[0][1], c = m[0][2], d = m[1][0], e = m[1][1], f = m[1][2], g = m[2][0],
                     h = m[2][1], k = m[2][2];
        const double A = e * k - f * h, B = -(d * k - f * g), C = d * h - e * g;
        const double det = a * A + b * B + c * C;
        Matrix3 r;
        r.m[0][0] = A / det; r.m[0][1] = -(b * k - c * h) / det; r.m[0][2] = (b * f - c * e) / det;
        r.m[1][0] = B / det; r.m[1][1] = (a * k - c * g) / det; r.m[1][2] = -(a * f - c * d) / det;
        r.m[2][0] = C / det; r.m[2][1] = -(a * h - b * g) / det; r.m[2][2] = (a * e - b * d) / det;
        return r;
    }
};
inline Vector3 operator*(const Matrix3& a, const Vector3& x)
{
    Vector3 r;
    for (int h = 0; h < 3; ++h) r.v[h] = a.m[h][0] * x.v[0] + a.m[h][1] * x.v[1] + a.m[h][2] * x.v[2];
    return r;
}

struct Matrix4 {
    double m[4][4];
    Matrix4() { for (int h = 0; h < 4; ++h) for (int k = 0; k < 4; ++k) m[h][k] = 0.0; }
    double& operator()(int h, int k) { return m[h][k]; }
    double operator()(int h, int k) const { return m[h][k]; }
};

namespace Eigen {
typedef ::Vector3 Vector3d;
typedef ::Vector2 Vector2d;
typedef ::Matrix3 Matrix3d;
typedef ::Matrix4 Matrix4d;
}  // namespace Eigen

enum eBoundaryTypes { eBound_FreeBound = -1, eBound_LockBound = -2, eBound_OutSource = -3, eBound_InnerSource = -4 };

struct Normals {
    std::vector<Vector3> n;
    Normals(const int size = base) { n.resize(size); }
};
struct Face {
    Vector3 A;
    Vector3 B;
    Vector3 C;
};
struct FaceCell {
    int face_id;
    Face face;
};
struct cell_local {
    Type s;
    Vector2 x0;
    ShortId in_face_id;
};
struct BasePointTetra {
    Vector3 x[base][NUMBER_OF_MEASUREMENTS];
    Vector3 operator()(const int i, const int j) const { return x[i][j]; }
};

#define check_bit(word, idx) ((word >> (idx)) & 0x1)
#define clear_bit(word, idx) (word & (~(1 << (idx))))
#define set_bit(word, idx) (word | (1 << (idx)))

const double eps = 1e-10;
#define PI 3.14159265358979323846
#define C_LIGHT 299792458.0
#define DIST 1e6
#define VELOCITY (3 * 1e8)
#define DENSITY (3.34 * 10e-14)
#define PRESSURE (DENSITY * VELOCITY * VELOCITY)
#define RADIATION (DENSITY * VELOCITY * VELOCITY * VELOCITY)
const Type R_gas = 8.314;
const Type c_light = C_LIGHT;
const Type h_plank = 6.62 * 1e-34;
const Type k_boltzmann = 1.38 * 1e-23;
const Type sigma_thomson = 6.652 * 1e-29;
const Type m_hydrogen = 1.6735575 * 1e-27;

struct flux_t {
    Type d;
    Vector3 v;
    Type p;
};
struct solve_mode_t {
    int class_vtk = 0;
};
static solve_mode_t solve_mode;
struct grid_t {
    int size;
    Type* Illum;
    Type* scattering;
};
static std::vector<flux_t> phys_local;

struct BaseTetra_t {
    Vector3 start_point_plane_coord;
    Matrix3 transform_matrix;
    Matrix3 inverse_transform_matrix;
    Matrix3 straight_face;
    Matrix3 inclined_face;
    Matrix3 straight_face_inverse;
    Matrix3 inclined_face_inverse;
    BaseTetra_t();
};

// The 2-D coordinates of the back-traced point on the in-face (x0 of
// cell_local) are not read by the sweep; the reference's computation of them
// (struct_short_characteristics_logic_function.cpp:75-220) needs a 4x4
// inverse and is left out.
static Vector2 CalculateIllumeOnInnerFace(const int, const int, const Matrix4&, const Vector3&, const Vector3&,
                                          std::vector<Type>&)
{
    return Vector2(0, 0);
}
