// cuda_solve.h (stand-in) -- the declarations of the reference's
// cuda/cuda_solve.h:5-37 over minimal stand-ins for the reference's types, so
// that cuda_solve_compat.cpp can be compiled and tested outside the
// reference tree.  Inside the reference build the real header is used.
//   grid_directions_t, direction_s ... global_def.h:79-90
//   grid_t ........................... solve_module/solve_global_struct.h:153-230
//                                      (ILLUM, USE_CUDA, ON_FULL_ILLUM_ARRAYS)
//   e_cuda_stream_id_t ............... solve_module/solve_global_struct.h:234-240
#pragma once
#include <vector>

typedef double Type;
#ifndef base
#define base 4
#endif

struct Vector3 {  // layout of Eigen::Vector3d: three contiguous doubles
    double v[3];
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
};
struct Matrix3 {  // layout of Eigen::Matrix3d: nine contiguous doubles
    double m[9];
};

struct direction_s {
    Vector3 dir;
    Type area;
};
struct grid_directions_t {
    int size;
    std::vector<direction_s> directions;
    Type full_area;
};

struct grid_t {
    int size = 0;
    Type* Illum = nullptr;
    Type* scattering = nullptr;
    Type* divstream = nullptr;
    Vector3* divimpuls = nullptr;
    Type* energy = nullptr;
    Vector3* stream = nullptr;
    Matrix3* impuls = nullptr;
};

enum e_cuda_stream_id_t { eCuda_scattering_1 = 0, eCuda_scattering_2, eCuda_params, eCuda_count };

void CudaEventPrint();
void CudaSyncStream(const e_cuda_stream_id_t stream_id);
int CalculateIntScatteringAsyncMPIStream(const grid_directions_t& grid_dir, grid_t& grid, const int start,
                                         const int end, const e_cuda_stream_id_t stream);
void CudaSendIllumAsync(const int size, const int shift, const Type* Illum_host);
void CudaSendIllumAsync(const int size, const int shift_dev, const int shift_host, const Type* Illum_host);
int CalculateIntScatteringAsyncMPI(const grid_directions_t& grid_dir, grid_t& grid, int local_size);
void CopyIllumOnDevice(const int size, const Type* Illum_host);
int CalculateIntScattering(const grid_directions_t& grid_dir, grid_t& grid);
int CalculateIntScatteringAsync(const grid_directions_t& grid_dir, grid_t& grid);
int CalculateEnergy(const grid_directions_t& grid_dir, grid_t& grid);
int CalculateStream(const grid_directions_t& grid_dir, grid_t& grid);
int CalculateImpuls(const grid_directions_t& grid_dir, grid_t& grid);
int CalculateDivImpuls(const grid_directions_t& grid_dir, grid_t& grid);
int CalculateDivStream(const grid_directions_t& grid_dir, grid_t& grid);
int CalculateAllParam(const grid_directions_t& grid_dir, grid_t& grid);
int CalculateAllParamStream(const grid_directions_t& grid_dir, grid_t& grid, e_cuda_stream_id_t st);
void SetDevice(const int num_dev);
void InitDevice(const grid_directions_t& grid_dir_host, grid_t& grid_host, const int start, const int end);
void ClearDevice();
void ClearHost(grid_t& grid_host);
void CudaWait();
