// Per-kernel drop-ins for the dimensionless reference kernels
// (Dimensionless/kernels_HT3D.jl, Dimensionless/HydroThermal3D_Alban_v6.jl,
// tools/Macros.jl) and the DYREL support kernels of
// Dimensional/kernels_HT3D_dimensional.jl.
//
// Each kernel evaluates the reference statements with ParallelStencil's
// semantics: every `@all(X) = ...` is guarded by X's own extent and the
// statements of one kernel run in order per grid point.  These are the
// granular, reference-shaped entry points; the fused solver in dyrel.cu is the
// fast path.
#include "ht3d_internal.cuh"

#define GIDX                                                \
    const int i = blockIdx.x * blockDim.x + threadIdx.x;    \
    const int j = blockIdx.y * blockDim.y + threadIdx.y;    \
    const int k = blockIdx.z * blockDim.z + threadIdx.z

// index helpers for the staggered shapes
#define CX(a, i, j, k) a[ix3(i, j, k, nx, ny)]                  // cell
#define EX(a, i, j, k) a[ix3(i, j, k, nx + 2, ny + 2)]          // ghosted
#define FX(a, i, j, k) a[ix3(i, j, k, nx + 1, ny)]              // x-face
#define FY(a, i, j, k) a[ix3(i, j, k, nx, ny + 1)]              // y-face
#define FZ(a, i, j, k) a[ix3(i, j, k, nx, ny)]                  // z-face (nx,ny,nz+1)
#define VX(a, i, j, k) a[ix3(i, j, k, nx + 1, ny + 1)]          // vertex

// ---------------------------------------------------------------- kernels
__global__ void k_init_vel(double* Vx, double* Vy, double* Vz, const double* __restrict__ kx,
                           const double* __restrict__ ky, const double* __restrict__ kz, const double* __restrict__ P,
                           const double* __restrict__ Ty, double Ra, double _dx, double _dy, double _dz, int nx,
                           int ny, int nz) {
    GIDX;
    if (i < nx + 1 && j < ny && k < nz)
        FX(Vx, i, j, k) = -FX(kx, i, j, k) * _dx * (EX(P, i + 1, j + 1, k + 1) - EX(P, i, j + 1, k + 1));
    if (i < nx && j < ny + 1 && k < nz)
        FY(Vy, i, j, k) = -FY(ky, i, j, k) * (_dy * (EX(P, i + 1, j + 1, k + 1) - EX(P, i + 1, j, k + 1)) - Ra * FY(Ty, i, j, k));
    if (i < nx && j < ny && k < nz + 1)
        FZ(Vz, i, j, k) = -FZ(kz, i, j, k) * _dz * (EX(P, i + 1, j + 1, k + 1) - EX(P, i + 1, j + 1, k));
}

// kx = av_yza(kv), ky = av_xza(kv), kz = av_xya(kv)
__device__ __forceinline__ void faces_from_vertices(double* kx, double* ky, double* kz, const double* __restrict__ kv,
                                                    int i, int j, int k, int nx, int ny, int nz) {
    if (i < nx + 1 && j < ny && k < nz)
        FX(kx, i, j, k) = (VX(kv, i, j, k) + VX(kv, i, j + 1, k) + VX(kv, i, j, k + 1) + VX(kv, i, j + 1, k + 1)) * 0.25;
    if (i < nx && j < ny + 1 && k < nz)
        FY(ky, i, j, k) = (VX(kv, i, j, k) + VX(kv, i + 1, j, k) + VX(kv, i, j, k + 1) + VX(kv, i + 1, j, k + 1)) * 0.25;
    if (i < nx && j < ny && k < nz + 1)
        FZ(kz, i, j, k) = (VX(kv, i, j, k) + VX(kv, i + 1, j, k) + VX(kv, i, j + 1, k) + VX(kv, i + 1, j + 1, k)) * 0.25;
}

__global__ void k_init_darcy(double* Ty, double* kx, double* ky, double* kz, const double* __restrict__ T,
                             const double* __restrict__ kv, int nx, int ny, int nz) {
    GIDX;
    if (i < nx && j < ny + 1 && k < nz) FY(Ty, i, j, k) = (EX(T, i + 1, j, k + 1) + EX(T, i + 1, j + 1, k + 1)) * 0.5;
    faces_from_vertices(kx, ky, kz, kv, i, j, k, nx, ny, nz);
}

__global__ void k_init_thermal(double* Rt, double* kx, double* ky, double* kz, const double* __restrict__ T,
                               const double* __restrict__ kv, double _dt, int nx, int ny, int nz) {
    GIDX;
    if (i < nx && j < ny && k < nz) CX(Rt, i, j, k) = -_dt * EX(T, i + 1, j + 1, k + 1);
    faces_from_vertices(kx, ky, kz, kv, i, j, k, nx, ny, nz);
}

__global__ void k_compute_rp(double* Rp, const double* __restrict__ ky, const double* __restrict__ Ty, double Ra,
                             double _dy, int nx, int ny, int nz) {
    GIDX;
    if (i < nx && j < ny && k < nz)
        CX(Rp, i, j, k) = Ra * _dy * ((FY(ky, i, j + 1, k) * FY(Ty, i, j + 1, k)) - (FY(ky, i, j, k) * FY(Ty, i, j, k)));
}

__global__ void k_compute_flux(double* qx, double* qy, double* qz, const double* __restrict__ kx,
                               const double* __restrict__ ky, const double* __restrict__ kz, const double* __restrict__ A,
                               double _dx, double _dy, double _dz, int nx, int ny, int nz) {
    GIDX;
    if (i < nx + 1 && j < ny && k < nz)
        FX(qx, i, j, k) = -FX(kx, i, j, k) * (_dx * (EX(A, i + 1, j + 1, k + 1) - EX(A, i, j + 1, k + 1)));
    if (i < nx && j < ny + 1 && k < nz)
        FY(qy, i, j, k) = -FY(ky, i, j, k) * (_dy * (EX(A, i + 1, j + 1, k + 1) - EX(A, i + 1, j, k + 1)));
    if (i < nx && j < ny && k < nz + 1)
        FZ(qz, i, j, k) = -FZ(kz, i, j, k) * (_dz * (EX(A, i + 1, j + 1, k + 1) - EX(A, i + 1, j + 1, k)));
}

__device__ __forceinline__ double div_q(const double* __restrict__ qx, const double* __restrict__ qy,
                                        const double* __restrict__ qz, double _dx, double _dy, double _dz, int i,
                                        int j, int k, int nx, int ny, int nz) {
    return _dx * (FX(qx, i + 1, j, k) - FX(qx, i, j, k)) + _dy * (FY(qy, i, j + 1, k) - FY(qy, i, j, k)) +
           _dz * (FZ(qz, i, j, k + 1) - FZ(qz, i, j, k));
}

// mode 0: UpdateT!, 1: ResidualDiffusion!, 2: ResidualDiffusionTransient!
template <int MODE>
__global__ void k_residual(double* F, double* T, const double* __restrict__ R, const double* __restrict__ qx,
                           const double* __restrict__ qy, const double* __restrict__ qz, double _dt, double dtau,
                           double _dx, double _dy, double _dz, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const double q = div_q(qx, qy, qz, _dx, _dy, _dz, i, j, k, nx, ny, nz);
    if (MODE == 1) {
        CX(F, i, j, k) = CX(R, i, j, k) + _dx * (FX(qx, i + 1, j, k) - FX(qx, i, j, k)) +
                         _dy * (FY(qy, i, j + 1, k) - FY(qy, i, j, k)) + _dz * (FZ(qz, i, j, k + 1) - FZ(qz, i, j, k));
        (void)q;
        return;
    }
    const double Tc = EX(T, i + 1, j + 1, k + 1);
    const double f = CX(R, i, j, k) + _dt * Tc + _dx * (FX(qx, i + 1, j, k) - FX(qx, i, j, k)) +
                     _dy * (FY(qy, i, j + 1, k) - FY(qy, i, j, k)) + _dz * (FZ(qz, i, j, k + 1) - FZ(qz, i, j, k));
    CX(F, i, j, k) = f;
    if (MODE == 0) EX(T, i + 1, j + 1, k + 1) = Tc - dtau * f;
}

// mode 0: UpdateP!/DampedUpdate! (F0 = F + a*F0), 1: DYRELUpdate! (F0 = a*F0 + b*F)
template <int MODE>
__global__ void k_update(double* F0, double* X, const double* __restrict__ F, double a, double b, double dtau, int nx,
                         int ny, int nz) {
    for_cells_z(nx, ny, nz, [&](int i, int j, int k) {
        const double f0 = MODE == 0 ? CX(F, i, j, k) + a * CX(F0, i, j, k) : a * CX(F0, i, j, k) + b * CX(F, i, j, k);
        CX(F0, i, j, k) = f0;
        EX(X, i + 1, j + 1, k + 1) = EX(X, i + 1, j + 1, k + 1) - dtau * f0;
    });
}

// Six-face ghost rules of the dimensionless BC kernels, with snapshot
// semantics (every rule reads other cells as they were before the launch;
// later rules of one ghost overwrite earlier ones).  The launch is split in
// three phases so no thread reads a cell another thread of the same launch
// writes: corners (read edge ghosts), then edges (read face ghosts), then
// face ghosts (read inner cells).  Each phase runs over the ghost shell only:
// thread t walks the planes x-, x+, y-, y+, z-, z+ in turn, and a cell on
// several planes (an edge or a corner) belongs to the first of them.
struct FaceBC {
    int type[6];
    double val[6];
};
__device__ __forceinline__ double bc_rule(const FaceBC& bc, int f, double inner) {
    return bc.type[f] == HT3D_BC_DIRICHLET ? 2.0 * bc.val[f] - inner : inner;
}
__global__ void k_face_bc(double* X, FaceBC bc, int phase, int nx, int ny, int nz) {
    const int n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    const long long px = (long long)n2 * n3, py = (long long)n1 * n3, pz = (long long)n1 * n2;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int i, j, k;
    if (t < 2 * px) {
        i = t < px ? 0 : n1 - 1;
        const long long r = t % px;
        j = (int)(r % n2);
        k = (int)(r / n2);
    } else if (t < 2 * (px + py)) {
        t -= 2 * px;
        j = t < py ? 0 : n2 - 1;
        const long long r = t % py;
        i = (int)(r % n1);
        k = (int)(r / n1);
        if (i == 0 || i == n1 - 1) return;  // on an x plane
    } else if (t < 2 * (px + py + pz)) {
        t -= 2 * (px + py);
        k = t < pz ? 0 : n3 - 1;
        const long long r = t % pz;
        i = (int)(r % n1);
        j = (int)(r / n1);
        if (i == 0 || i == n1 - 1 || j == 0 || j == n2 - 1) return;  // on an x or y plane
    } else {
        return;
    }
    const int nb = (i == 0 || i == n1 - 1) + (j == 0 || j == n2 - 1) + (k == 0 || k == n3 - 1);
    if (nb == 0 || (3 - nb) != phase) return;  // phase 0: corners (nb=3), 1: edges, 2: faces
    double v = 0.0;
    bool set = false;
    if (i == 0) { v = bc_rule(bc, 0, X[ix3(1, j, k, n1, n2)]); set = true; }
    if (i == n1 - 1) { v = bc_rule(bc, 1, X[ix3(n1 - 2, j, k, n1, n2)]); set = true; }
    if (j == 0) { v = bc_rule(bc, 2, X[ix3(i, 1, k, n1, n2)]); set = true; }
    if (j == n2 - 1) { v = bc_rule(bc, 3, X[ix3(i, n2 - 2, k, n1, n2)]); set = true; }
    if (k == 0) { v = bc_rule(bc, 4, X[ix3(i, j, 1, n1, n2)]); set = true; }
    if (k == n3 - 1) { v = bc_rule(bc, 5, X[ix3(i, j, n3 - 2, n1, n2)]); set = true; }
    if (set) X[ix3(i, j, k, n1, n2)] = v;
}

// one thread per (i, k) column zeroes the south (j = 0) and north (j = ny) faces
__global__ void k_kill_ns(double* Ty, int nx, int ny, int nz) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nx * nz) return;
    const int i = (int)(t % nx), k = (int)(t / nx);
    FY(Ty, i, 0, k) = 0.0;
    FY(Ty, i, ny, k) = 0.0;
}

__global__ void k_reset2(double* A, double* B, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        A[t] = 0.0;
        B[t] = 0.0;
    }
}
__global__ void k_copy(double* A, const double* __restrict__ B, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        A[t] = B[t];
}
__global__ void k_mul(double* a, const double* __restrict__ b, const double* __restrict__ c, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        a[t] = b[t] * c[t];
}
// dir 0: A(n^3) = inn(B), 1: inn(A) = B(n^3)
template <int DIR>
__global__ void k_cpy_inn(double* A, const double* __restrict__ B, int nx, int ny, int nz) {
    for_cells_z(nx, ny, nz, [&](int i, int j, int k) {
        if (DIR == 0) CX(A, i, j, k) = EX(B, i + 1, j + 1, k + 1);
        else EX(A, i + 1, j + 1, k + 1) = CX(B, i, j, k);
    });
}

// GershgorinPoisson!  Dimensional/kernels_HT3D_dimensional.jl:207-221
// (HYDRO = 1: GershgorinHydro! :335-347, G only, no division)
template <int HYDRO>
__global__ void k_gershgorin(double* G, double* D, const double* __restrict__ rC, const double* __restrict__ kx,
                             const double* __restrict__ ky, const double* __restrict__ kz, double transient, double dt,
                             double dx, double dy, double dz, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const double kW = FX(kx, i, j, k), kE = FX(kx, i + 1, j, k), kS = FY(ky, i, j, k), kN = FY(ky, i, j + 1, k),
                 kF = FZ(kz, i, j, k + 1), kB = FZ(kz, i, j, k), rhoC = CX(rC, i, j, k);
    const double diag = ((kB / dz + kF / dz) / dz + (kN / dy + kS / dy) / dy + (kE / dx + kW / dx) / dx + rhoC * transient / dt);
    double g = fabs(kE / (dx * dx)) + fabs(kW / (dx * dx)) + fabs(kN / (dy * dy)) + fabs(kS / (dy * dy)) +
               fabs(kB / (dz * dz)) + fabs(kF / (dz * dz)) + fabs(diag);
    if (HYDRO) {
        CX(G, i, j, k) = g;
        return;
    }
    CX(D, i, j, k) = diag;
    CX(G, i, j, k) = g / diag;
}

__global__ void k_swap_dyrel(double* Xc, double* Yc, const double* __restrict__ X0, const double* __restrict__ Y0,
                             int nx, int ny, int nz) {
    for_cells_z(nx, ny, nz, [&](int i, int j, int k) {
        CX(Xc, i, j, k) = EX(X0, i + 1, j + 1, k + 1);
        CX(Yc, i, j, k) = CX(Y0, i, j, k);
    });
}

template <int DEN>
__global__ void k_rayleigh(double* G, const double* __restrict__ F0, const double* __restrict__ Fit,
                           const double* __restrict__ F, double dtau, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double d = dtau * F0[t];
        G[t] = DEN ? d * d : -d * (F[t] - Fit[t]);
    }
}

// ---------------------------------------------------------------- launchers
static inline dim3 g1(ht3d_ctx* ctx, long long n) {
    long long b = (n + 255) / 256;
    return dim3((unsigned)std::max<long long>(1, std::min<long long>(b, (long long)ctx->num_sms * 16)));
}

void ht3d_launch_face_bc(ht3d_ctx* ctx, double* X, const int* type6, const double* val6, int nx, int ny, int nz) {
    FaceBC bc;
    for (int f = 0; f < 6; ++f) {
        HT3D_REQUIRE(type6[f] == HT3D_BC_NEUMANN || type6[f] == HT3D_BC_DIRICHLET, "face BC type must be 0 or 1");
        bc.type[f] = type6[f];
        bc.val[f] = val6[f];
    }
    const long long n1 = nx + 2, n2 = ny + 2, n3 = nz + 2, shell = 2 * (n2 * n3 + n1 * n3 + n1 * n2);
    const unsigned blocks = (unsigned)((shell + 255) / 256);
    for (int ph = 0; ph < 3; ++ph) HT3D_LAUNCH(ctx, k_face_bc, dim3(blocks), dim3(256), 0, X, bc, ph, nx, ny, nz);
}

extern "C" {

#define DIMS_OK(minn) ht3d_check_dims(nx, ny, nz, minn)
#define G3(a, b, c) grid3((a), (b), (c), kBlock3)

int ht3d_Init_vel(ht3d_ctx* ctx, double* Vx, double* Vy, double* Vz, const double* kx, const double* ky,
                  const double* kz, const double* Pc_ex, const double* Ty, double Ra, double _dx, double _dy,
                  double _dz, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_init_vel, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty, Ra,
                    _dx, _dy, _dz, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_InitDarcy(ht3d_ctx* ctx, double* Ty, double* kx, double* ky, double* kz, const double* Tc_ex,
                   const double* kfv, double _dt, int nx, int ny, int nz) {
    (void)_dt;
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Ty, kx, ky, kz, Tc_ex, kfv), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_init_darcy, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, Ty, kx, ky, kz, Tc_ex, kfv, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_Compute_Rp(ht3d_ctx* ctx, double* Rp, const double* ky, const double* Ty, double Ra, double _dy, int nx,
                    int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Rp, ky, Ty), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_compute_rp, G3(nx, ny, nz), kBlock3, 0, Rp, ky, Ty, Ra, _dy, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_InitThermal(ht3d_ctx* ctx, double* Rt, double* kx, double* ky, double* kz, const double* Tc_ex,
                     const double* ktv, double _dt, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Rt, kx, ky, kz, Tc_ex, ktv), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_init_thermal, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, Rt, kx, ky, kz, Tc_ex, ktv, _dt, nx,
                    ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ComputeFlux(ht3d_ctx* ctx, double* qx, double* qy, double* qz, const double* kx, const double* ky,
                     const double* kz, const double* A, double _dx, double _dy, double _dz, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(qx, qy, qz, kx, ky, kz, A), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_compute_flux, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, qx, qy, qz, kx, ky, kz, A, _dx, _dy,
                    _dz, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_UpdateT(ht3d_ctx* ctx, double* F, double* T, const double* R, const double* qx, const double* qy,
                 const double* qz, double _dt, double dtau, double _dx, double _dy, double _dz, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(F, T, R, qx, qy, qz), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_residual<0>, G3(nx, ny, nz), kBlock3, 0, F, T, R, qx, qy, qz, _dt, dtau, _dx, _dy, _dz, nx,
                    ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ResidualDiffusion(ht3d_ctx* ctx, double* F, const double* R, const double* qx, const double* qy,
                           const double* qz, double _dx, double _dy, double _dz, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(F, R, qx, qy, qz), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_residual<1>, G3(nx, ny, nz), kBlock3, 0, F, (double*)nullptr, R, qx, qy, qz, 0.0, 0.0, _dx,
                    _dy, _dz, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ResidualDiffusionTransient(ht3d_ctx* ctx, double* F, const double* T, const double* R, const double* qx,
                                    const double* qy, const double* qz, double _dt, double _dx, double _dy,
                                    double _dz, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(F, T, R, qx, qy, qz), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_residual<2>, G3(nx, ny, nz), kBlock3, 0, F, (double*)T, R, qx, qy, qz, _dt, 0.0, _dx, _dy,
                    _dz, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_UpdateP(ht3d_ctx* ctx, double* F0, double* P, const double* F, double dampx, double dtau, int nx, int ny,
                 int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(F0, P, F), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_update<0>, grid3z(nx, ny, nz), kBlock3, 0, F0, P, F, dampx, 0.0, dtau, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_DYRELUpdate(ht3d_ctx* ctx, double* F0, double* X, const double* F, double h1, double h2, double dtau,
                     int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(F0, X, F), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_update<1>, grid3z(nx, ny, nz), kBlock3, 0, F0, X, F, h1, h2, dtau, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_SetFaceBCs(ht3d_ctx* ctx, double* X_ex, const int* bc_type6, const double* bc_val6, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        DIMS_OK(1);
        HT3D_REQUIRE(X_ex && bc_type6 && bc_val6, "null argument");
        ht3d_launch_face_bc(ctx, X_ex, bc_type6, bc_val6, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_SetPressureBCs(ht3d_ctx* ctx, double* Pc_ex, double Pbot, double Ptop, int nx, int ny, int nz) {
    const int t[6] = {HT3D_BC_NEUMANN, HT3D_BC_NEUMANN, HT3D_BC_DIRICHLET, HT3D_BC_DIRICHLET, HT3D_BC_NEUMANN, HT3D_BC_NEUMANN};
    const double v[6] = {0.0, 0.0, Pbot, Ptop, 0.0, 0.0};
    return ht3d_SetFaceBCs(ctx, Pc_ex, t, v, nx, ny, nz);
}

int ht3d_KillNorthSouthFluxes(ht3d_ctx* ctx, double* Ty, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Ty), "null argument");
        DIMS_OK(1);
        const long long cols = (long long)nx * nz;
        HT3D_LAUNCH(ctx, k_kill_ns, dim3((unsigned)((cols + 255) / 256)), dim3(256), 0, Ty, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ResetA(ht3d_ctx* ctx, double* A, double* B, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(A, B), "null argument");
        HT3D_REQUIRE(n >= 0, "negative size");
        if (n) HT3D_LAUNCH(ctx, k_reset2, g1(ctx, n), 256, 0, A, B, n);
        return HT3D_OK;
    });
}

int ht3d_Cpy_inn_to_all(ht3d_ctx* ctx, double* A, const double* B_ex, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(A, B_ex), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_cpy_inn<0>, grid3z(nx, ny, nz), kBlock3, 0, A, B_ex, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_Cpy_all_to_inn(ht3d_ctx* ctx, double* A_ex, const double* B, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(A_ex, B), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_cpy_inn<1>, grid3z(nx, ny, nz), kBlock3, 0, A_ex, B, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ArrayEqualArray(ht3d_ctx* ctx, double* A, const double* B, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(A, B), "null argument");
        HT3D_REQUIRE(n >= 0, "negative size");
        if (n) HT3D_LAUNCH(ctx, k_copy, g1(ctx, n), 256, 0, A, B, n);
        return HT3D_OK;
    });
}

int ht3d_Multiply(ht3d_ctx* ctx, double* a, const double* b, const double* c, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(a, c), "null argument");
        HT3D_REQUIRE(n >= 0, "negative size");
        if (n) HT3D_LAUNCH(ctx, k_mul, g1(ctx, n), 256, 0, a, b, c, n);
        return HT3D_OK;
    });
}

int ht3d_GershgorinPoisson(ht3d_ctx* ctx, double* G, double* D, const double* rhoC_eff, const double* kx,
                           const double* ky, const double* kz, double transient, double dt, double dx, double dy,
                           double dz, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(G, D, rhoC_eff, kx, ky, kz), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_gershgorin<0>, G3(nx, ny, nz), kBlock3, 0, G, D, rhoC_eff, kx, ky, kz, transient, dt, dx, dy,
                    dz, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_GershgorinHydro(ht3d_ctx* ctx, double* G, const double* phidrhodP, const double* kx, const double* ky,
                         const double* kz, double transient, double dt, double dx, double dy, double dz, int nx,
                         int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(G, phidrhodP, kx, ky, kz), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_gershgorin<1>, G3(nx, ny, nz), kBlock3, 0, G, (double*)nullptr, phidrhodP, kx, ky, kz,
                    transient, dt, dx, dy, dz, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_SwapDYREL(ht3d_ctx* ctx, double* Xc, double* Yc, const double* X0c_ex, const double* Y0c, int nx, int ny,
                   int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Xc, Yc, X0c_ex, Y0c), "null argument");
        DIMS_OK(1);
        HT3D_LAUNCH(ctx, k_swap_dyrel, grid3z(nx, ny, nz), kBlock3, 0, Xc, Yc, X0c_ex, Y0c, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_RayleighQuotientNumerator(ht3d_ctx* ctx, double* G, const double* Fc0, const double* Fcit, const double* Fc,
                                   double dtau, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(G, Fc0, Fcit, Fc), "null argument");
        HT3D_REQUIRE(n >= 0, "negative size");
        if (n) HT3D_LAUNCH(ctx, k_rayleigh<0>, g1(ctx, n), 256, 0, G, Fc0, Fcit, Fc, dtau, n);
        return HT3D_OK;
    });
}

int ht3d_RayleighQuotientDenominator(ht3d_ctx* ctx, double* G, const double* Fc0, double dtau, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(G, Fc0), "null argument");
        HT3D_REQUIRE(n >= 0, "negative size");
        if (n) HT3D_LAUNCH(ctx, k_rayleigh<1>, g1(ctx, n), 256, 0, G, Fc0, (const double*)nullptr, (const double*)nullptr, dtau, n);
        return HT3D_OK;
    });
}

}  // extern "C"
