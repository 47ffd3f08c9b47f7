// Kernels of the dimensionless HRL time step (Dimensionless/kernels_HT3D.jl
// and Dimensionless/HydroThermal3D_Alban_v6.jl), shared by the single-instance
// step (step.cu) and the ensemble step (ensemble.cu).  Both translation units
// are compiled without FMA contraction, so the two produce identical bits.
#pragma once
#include "ht3d_internal.cuh"

namespace {

#define GIDX                                             \
    const int i = blockIdx.x * blockDim.x + threadIdx.x; \
    const int j = blockIdx.y * blockDim.y + threadIdx.y; \
    const int k = blockIdx.z * blockDim.z + threadIdx.z

__device__ __forceinline__ void faces_from_vertices(double* kx, double* ky, double* kz, const double* __restrict__ kv,
                                                    int i, int j, int k, int nx, int ny, int nz) {
    const int v1 = nx + 1, v2 = ny + 1;
    if (i < nx + 1 && j < ny && k < nz)
        kx[ix3(i, j, k, nx + 1, ny)] = (kv[ix3(i, j, k, v1, v2)] + kv[ix3(i, j + 1, k, v1, v2)] +
                                        kv[ix3(i, j, k + 1, v1, v2)] + kv[ix3(i, j + 1, k + 1, v1, v2)]) * 0.25;
    if (i < nx && j < ny + 1 && k < nz)
        ky[ix3(i, j, k, nx, ny + 1)] = (kv[ix3(i, j, k, v1, v2)] + kv[ix3(i + 1, j, k, v1, v2)] +
                                        kv[ix3(i, j, k + 1, v1, v2)] + kv[ix3(i + 1, j, k + 1, v1, v2)]) * 0.25;
    if (i < nx && j < ny && k < nz + 1)
        kz[ix3(i, j, k, nx, ny)] = (kv[ix3(i, j, k, v1, v2)] + kv[ix3(i + 1, j, k, v1, v2)] +
                                    kv[ix3(i, j + 1, k, v1, v2)] + kv[ix3(i + 1, j + 1, k, v1, v2)]) * 0.25;
}

// InitThermal! (Dimensionless/kernels_HT3D.jl:99-107)
__global__ void k_step_init_thermal(double* Rt, double* kx, double* ky, double* kz, const double* __restrict__ T,
                                    const double* __restrict__ kv, double _dt, int nx, int ny, int nz) {
    GIDX;
    if (i < nx && j < ny && k < nz) Rt[ix3(i, j, k, nx, ny)] = -_dt * T[ix3(i + 1, j + 1, k + 1, nx + 2, ny + 2)];
    faces_from_vertices(kx, ky, kz, kv, i, j, k, nx, ny, nz);
}

// InitDarcy! + KillNorthSouthFluxes! (Alban_v6.jl:47-55, 153-159)
__global__ void k_step_init_darcy(double* Ty, double* kx, double* ky, double* kz, const double* __restrict__ T,
                                  const double* __restrict__ kv, int kill_ns, int nx, int ny, int nz) {
    GIDX;
    if (i < nx && j < ny + 1 && k < nz) {
        double t = (T[ix3(i + 1, j, k + 1, nx + 2, ny + 2)] + T[ix3(i + 1, j + 1, k + 1, nx + 2, ny + 2)]) * 0.5;
        if (kill_ns && (j == 0 || j == ny)) t = 0.0;
        Ty[ix3(i, j, k, nx, ny + 1)] = t;
    }
    faces_from_vertices(kx, ky, kz, kv, i, j, k, nx, ny, nz);
}

// Compute_Rp! (Dimensionless/kernels_HT3D.jl:92-97)
__global__ void k_step_rp(double* Rp, const double* __restrict__ ky, const double* __restrict__ Ty, double Ra, double _dy,
                          int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const int a = ix3(i, j, k, nx, ny + 1), b = ix3(i, j + 1, k, nx, ny + 1);
    Rp[ix3(i, j, k, nx, ny)] = Ra * _dy * ((ky[b] * Ty[b]) - (ky[a] * Ty[a]));
}

// Init_vel! (Dimensionless/kernels_HT3D.jl:73-80)
__global__ void k_step_vel(double* Vx, double* Vy, double* Vz, const double* __restrict__ kx,
                           const double* __restrict__ ky, const double* __restrict__ kz, const double* __restrict__ P,
                           const double* __restrict__ Ty, double Ra, double _dx, double _dy, double _dz, int nx, int ny,
                           int nz) {
    GIDX;
    const int e1 = nx + 2, e2 = ny + 2;
    if (i < nx + 1 && j < ny && k < nz) {
        const int f = ix3(i, j, k, nx + 1, ny);
        Vx[f] = -kx[f] * _dx * (P[ix3(i + 1, j + 1, k + 1, e1, e2)] - P[ix3(i, j + 1, k + 1, e1, e2)]);
    }
    if (i < nx && j < ny + 1 && k < nz) {
        const int f = ix3(i, j, k, nx, ny + 1);
        Vy[f] = -ky[f] * (_dy * (P[ix3(i + 1, j + 1, k + 1, e1, e2)] - P[ix3(i + 1, j, k + 1, e1, e2)]) - Ra * Ty[f]);
    }
    if (i < nx && j < ny && k < nz + 1) {
        const int f = ix3(i, j, k, nx, ny);
        Vz[f] = -kz[f] * _dz * (P[ix3(i + 1, j + 1, k + 1, e1, e2)] - P[ix3(i + 1, j + 1, k, e1, e2)]);
    }
}

}  // namespace
