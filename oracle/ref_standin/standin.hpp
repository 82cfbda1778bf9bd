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
//   grid_t .................... solve_module/solve_global_struct.h:153-230
//                               (only size, Illum, scattering)
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

struct direction_s { Vector3 dir; Type area; };
struct grid_directions_t { int size; std::vector<direction_s> directions; Type full_area; };
struct grid_t { int size; Type* Illum; Type* scattering; };

#define MPI_GET_INF(np, myid) { np = 1; myid = 0; }

static std::vector<int> send_count;
static std::vector<int> disp;
