// ============================================================================
// ht3d oracle -- TEST INFRASTRUCTURE ONLY.
//
// A plain C++17 FP64 CPU restatement of the HydroThermal3D pseudo-transient
// hot path (tduretz/HydroThermal3D, Julia + ParallelStencil).  It exists only
// to check the CUDA library: the parity tests, __graft_entry__.smoke() and the
// bench's cpu_baseline / reference arm call it.  No product code path may link
// or call it.
//
// Parity status: the reference is Julia and cannot run here (no Julia, and the
// ParallelStencil version is unpinned), so this oracle is pinned against
//   * the known answers in the reference's own test scripts and notebook
//     (tools/TestAdvection.jl:84-116 Gaussian translation;
//      notebooks/Gershgorin_TH3D.ipynb cells 2 and 4),
//   * analytic properties (exact discrete steady states, conservation), and
//   * an independent numpy restatement written in the reference's array-slice
//     form (tests/golden/make_golden.py -> tests/golden/*.npz).
// It is NOT pinned against outputs of the running reference.
//
// Conventions
//   * Arrays are column-major, x fastest, exactly like Julia's Data.Array.
//     Index (i,j,k) here is 0-based: Julia A[i+1,j+1,k+1] == A(i,j,k).
//   * nx,ny,nz are numbers of cells.  Shapes: cell n^3, ghosted "ex" (n+2)^3,
//     WENO "exxx" (n+6)^3, x-faces (nx+1,ny,nz), y-faces (nx,ny+1,nz),
//     z-faces (nx,ny,nz+1), vertices (n+1)^3, wN (nx+2,nz+2).
//   * ParallelStencil semantics: every `@all(X) = ...` statement is guarded by
//     X's own extent, `@inn(X) = ...` by extent-2; statements of one kernel run
//     in order per grid point.
//   * Boundary-condition kernels write ghost cells in place.  The oracle fixes
//     the reference's inter-thread races with snapshot semantics: every rule
//     reads other cells as they were before the launch, and later rules of one
//     grid point overwrite earlier ones.  (Face ghosts never depend on this
//     choice; only edge/corner ghosts can.)
//   * Built with -ffp-contract=off so every rounding follows the source.
// ============================================================================
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>
#include "../hydrothermal3d_gb300/csrc/expo.h"

typedef long long i64;

struct A3 {
    double* p; i64 n1, n2, n3;
    inline double& operator()(i64 i, i64 j, i64 k) const { return p[i + n1 * (j + n2 * k)]; }
    i64 size() const { return n1 * n2 * n3; }
};
static inline A3 mk(double* p, i64 a, i64 b, i64 c) { return A3{p, a, b, c}; }
struct A2 {
    double* p; i64 n1, n2;
    inline double& operator()(i64 i, i64 k) const { return p[i + n1 * k]; }
};

#define PARFOR3(N1, N2, N3) \
    _Pragma("omp parallel for schedule(static)") \
    for (i64 k = 0; k < (N3); ++k) for (i64 j = 0; j < (N2); ++j) for (i64 i = 0; i < (N1); ++i)

// ---------------------------------------------------------------------------
// ParallelStencil FiniteDifferences3D macros (0-based restatement).
// ---------------------------------------------------------------------------
#define D_XA(A) (A(i + 1, j, k) - A(i, j, k))
#define D_YA(A) (A(i, j + 1, k) - A(i, j, k))
#define D_ZA(A) (A(i, j, k + 1) - A(i, j, k))
#define D_XI(A) (A(i + 1, j + 1, k + 1) - A(i, j + 1, k + 1))
#define D_YI(A) (A(i + 1, j + 1, k + 1) - A(i + 1, j, k + 1))
#define D_ZI(A) (A(i + 1, j + 1, k + 1) - A(i + 1, j + 1, k))
#define INN(A) A(i + 1, j + 1, k + 1)
#define AV(A) ((A(i, j, k) + A(i + 1, j, k) + A(i, j + 1, k) + A(i + 1, j + 1, k) + \
                A(i, j, k + 1) + A(i + 1, j, k + 1) + A(i, j + 1, k + 1) + A(i + 1, j + 1, k + 1)) * 0.125)
#define AV_XYA(A) ((A(i, j, k) + A(i + 1, j, k) + A(i, j + 1, k) + A(i + 1, j + 1, k)) * 0.25)
#define AV_XZA(A) ((A(i, j, k) + A(i + 1, j, k) + A(i, j, k + 1) + A(i + 1, j, k + 1)) * 0.25)
#define AV_YZA(A) ((A(i, j, k) + A(i, j + 1, k) + A(i, j, k + 1) + A(i, j + 1, k + 1)) * 0.25)
#define AV_YI(A) ((A(i + 1, j, k + 1) + A(i + 1, j + 1, k + 1)) * 0.5)
// tools/Macros.jl:111
#define DMUL_YA(A, B) ((A(i, j + 1, k) * B(i, j + 1, k)) - (A(i, j, k) * B(i, j, k)))

#define SHAPES                                                              \
    const i64 ex1 = nx + 2, ex2 = ny + 2, ex3 = nz + 2; (void)ex1; (void)ex2; (void)ex3; \
    (void)0

extern "C" {

int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_num_threads(int n) { if (n > 0) omp_set_num_threads(n); }

// ===========================================================================
// Dimensionless kernels (Dimensionless/kernels_HT3D.jl,
// Dimensionless/HydroThermal3D_Alban_v6.jl, tools/Macros.jl)
// ===========================================================================

// Init_vel!  Dimensionless/kernels_HT3D.jl:73-80
void orc_Init_vel(double* Vx_, double* Vy_, double* Vz_, const double* kx_, const double* ky_, const double* kz_,
                  const double* P_, const double* Ty_, double Ra, double _dx, double _dy, double _dz,
                  i64 nx, i64 ny, i64 nz) {
    A3 Vx = mk(Vx_, nx + 1, ny, nz), Vy = mk(Vy_, nx, ny + 1, nz), Vz = mk(Vz_, nx, ny, nz + 1);
    A3 kx = mk((double*)kx_, nx + 1, ny, nz), ky = mk((double*)ky_, nx, ny + 1, nz), kz = mk((double*)kz_, nx, ny, nz + 1);
    A3 P = mk((double*)P_, nx + 2, ny + 2, nz + 2), Ty = mk((double*)Ty_, nx, ny + 1, nz);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        if (i < nx + 1 && j < ny && k < nz) Vx(i, j, k) = -kx(i, j, k) * _dx * D_XI(P);
        if (i < nx && j < ny + 1 && k < nz) Vy(i, j, k) = -ky(i, j, k) * (_dy * D_YI(P) - Ra * Ty(i, j, k));
        if (i < nx && j < ny && k < nz + 1) Vz(i, j, k) = -kz(i, j, k) * _dz * D_ZI(P);
    }
}

// InitDarcy!  Dimensionless/kernels_HT3D.jl:82-90
void orc_InitDarcy(double* Ty_, double* kx_, double* ky_, double* kz_, const double* T_, const double* kfv_,
                   double _dt, i64 nx, i64 ny, i64 nz) {
    (void)_dt;
    A3 Ty = mk(Ty_, nx, ny + 1, nz), kx = mk(kx_, nx + 1, ny, nz), ky = mk(ky_, nx, ny + 1, nz), kz = mk(kz_, nx, ny, nz + 1);
    A3 T = mk((double*)T_, nx + 2, ny + 2, nz + 2), kv = mk((double*)kfv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        if (i < nx && j < ny + 1 && k < nz) Ty(i, j, k) = AV_YI(T);
        if (i < nx + 1 && j < ny && k < nz) kx(i, j, k) = AV_YZA(kv);
        if (i < nx && j < ny + 1 && k < nz) ky(i, j, k) = AV_XZA(kv);
        if (i < nx && j < ny && k < nz + 1) kz(i, j, k) = AV_XYA(kv);
    }
}

// Compute_Rp!  Dimensionless/kernels_HT3D.jl:92-97
void orc_Compute_Rp(double* Rp_, const double* ky_, const double* Ty_, double Ra, double _dy, i64 nx, i64 ny, i64 nz) {
    A3 Rp = mk(Rp_, nx, ny, nz), ky = mk((double*)ky_, nx, ny + 1, nz), Ty = mk((double*)Ty_, nx, ny + 1, nz);
    PARFOR3(nx, ny, nz) { Rp(i, j, k) = Ra * _dy * DMUL_YA(ky, Ty); }
}

// InitThermal!  Dimensionless/kernels_HT3D.jl:99-107
void orc_InitThermal_dimless(double* Rt_, double* kx_, double* ky_, double* kz_, const double* T_, const double* ktv_,
                             double _dt, i64 nx, i64 ny, i64 nz) {
    A3 Rt = mk(Rt_, nx, ny, nz), kx = mk(kx_, nx + 1, ny, nz), ky = mk(ky_, nx, ny + 1, nz), kz = mk(kz_, nx, ny, nz + 1);
    A3 T = mk((double*)T_, nx + 2, ny + 2, nz + 2), kv = mk((double*)ktv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        if (i < nx && j < ny && k < nz) Rt(i, j, k) = -_dt * INN(T);
        if (i < nx + 1 && j < ny && k < nz) kx(i, j, k) = AV_YZA(kv);
        if (i < nx && j < ny + 1 && k < nz) ky(i, j, k) = AV_XZA(kv);
        if (i < nx && j < ny && k < nz + 1) kz(i, j, k) = AV_XYA(kv);
    }
}

// ComputeFlux!  Dimensionless/kernels_HT3D.jl:109-117 (identical in
// Dimensional/kernels_HT3D_dimensional.jl:140-146)
void orc_ComputeFlux(double* qx_, double* qy_, double* qz_, const double* kx_, const double* ky_, const double* kz_,
                     const double* A_, double _dx, double _dy, double _dz, i64 nx, i64 ny, i64 nz) {
    A3 qx = mk(qx_, nx + 1, ny, nz), qy = mk(qy_, nx, ny + 1, nz), qz = mk(qz_, nx, ny, nz + 1);
    A3 kx = mk((double*)kx_, nx + 1, ny, nz), ky = mk((double*)ky_, nx, ny + 1, nz), kz = mk((double*)kz_, nx, ny, nz + 1);
    A3 A = mk((double*)A_, nx + 2, ny + 2, nz + 2);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        if (i < nx + 1 && j < ny && k < nz) qx(i, j, k) = -kx(i, j, k) * (_dx * D_XI(A));
        if (i < nx && j < ny + 1 && k < nz) qy(i, j, k) = -ky(i, j, k) * (_dy * D_YI(A));
        if (i < nx && j < ny && k < nz + 1) qz(i, j, k) = -kz(i, j, k) * (_dz * D_ZI(A));
    }
}

// UpdateT!  Dimensionless/kernels_HT3D.jl:119-126
void orc_UpdateT(double* F_, double* T_, const double* R_, const double* qx_, const double* qy_, const double* qz_,
                 double _dt, double dtau, double _dx, double _dy, double _dz, i64 nx, i64 ny, i64 nz) {
    A3 F = mk(F_, nx, ny, nz), T = mk(T_, nx + 2, ny + 2, nz + 2), R = mk((double*)R_, nx, ny, nz);
    A3 qx = mk((double*)qx_, nx + 1, ny, nz), qy = mk((double*)qy_, nx, ny + 1, nz), qz = mk((double*)qz_, nx, ny, nz + 1);
    PARFOR3(nx, ny, nz) {
        F(i, j, k) = R(i, j, k) + _dt * INN(T) + _dx * D_XA(qx) + _dy * D_YA(qy) + _dz * D_ZA(qz);
        INN(T) = INN(T) - dtau * F(i, j, k);
    }
}

// ResidualDiffusion!  Dimensionless/kernels_HT3D.jl:128-134
void orc_ResidualDiffusion(double* F_, const double* R_, const double* qx_, const double* qy_, const double* qz_,
                           double _dx, double _dy, double _dz, i64 nx, i64 ny, i64 nz) {
    A3 F = mk(F_, nx, ny, nz), R = mk((double*)R_, nx, ny, nz);
    A3 qx = mk((double*)qx_, nx + 1, ny, nz), qy = mk((double*)qy_, nx, ny + 1, nz), qz = mk((double*)qz_, nx, ny, nz + 1);
    PARFOR3(nx, ny, nz) { F(i, j, k) = R(i, j, k) + _dx * D_XA(qx) + _dy * D_YA(qy) + _dz * D_ZA(qz); }
}

// ResidualDiffusionTransient!  Dimensionless/HydroThermal3D_Alban_v6.jl:84-90
void orc_ResidualDiffusionTransient(double* F_, const double* T_, const double* R_, const double* qx_, const double* qy_,
                                    const double* qz_, double _dt, double _dx, double _dy, double _dz,
                                    i64 nx, i64 ny, i64 nz) {
    A3 F = mk(F_, nx, ny, nz), T = mk((double*)T_, nx + 2, ny + 2, nz + 2), R = mk((double*)R_, nx, ny, nz);
    A3 qx = mk((double*)qx_, nx + 1, ny, nz), qy = mk((double*)qy_, nx, ny + 1, nz), qz = mk((double*)qz_, nx, ny, nz + 1);
    PARFOR3(nx, ny, nz) {
        F(i, j, k) = R(i, j, k) + _dt * INN(T) + _dx * D_XA(qx) + _dy * D_YA(qy) + _dz * D_ZA(qz);
    }
}

// UpdateP!  Dimensionless/kernels_HT3D.jl:136-142; same body as
// DampedUpdate!  Dimensional/kernels_HT3D_dimensional.jl:316-320
void orc_UpdateP(double* F0_, double* P_, const double* F_, double dampx, double dtau, i64 nx, i64 ny, i64 nz) {
    A3 F0 = mk(F0_, nx, ny, nz), P = mk(P_, nx + 2, ny + 2, nz + 2), F = mk((double*)F_, nx, ny, nz);
    PARFOR3(nx, ny, nz) {
        F0(i, j, k) = F(i, j, k) + dampx * F0(i, j, k);
        INN(P) = INN(P) - dtau * F0(i, j, k);
    }
}

// DYRELUpdate!  Dimensional/kernels_HT3D_dimensional.jl:322-326
void orc_DYRELUpdate(double* F0_, double* X_, const double* F_, double h1, double h2, double dtau, i64 nx, i64 ny, i64 nz) {
    A3 F0 = mk(F0_, nx, ny, nz), X = mk(X_, nx + 2, ny + 2, nz + 2), F = mk((double*)F_, nx, ny, nz);
    PARFOR3(nx, ny, nz) {
        F0(i, j, k) = h1 * F0(i, j, k) + h2 * F(i, j, k);
        INN(X) = INN(X) - dtau * F0(i, j, k);
    }
}

// Generic face boundary conditions of the dimensionless drivers.
//   type 0 = Neumann (ghost = adjacent inner), type 1 = Dirichlet
//   (ghost = 2 v - adjacent inner).  Face order: W,E (x), S,N (y), B,F (z).
// Covers SetPressureBCs! Dimensionless/kernels_HT3D.jl:144-154 (x,z Neumann,
// y Dirichlet), SetTemperatureBCs!/SetPressureBCs! of
// Dimensionless/HydroThermal3D_Alban_v6.jl:108-130 (Dirichlet-y / all
// Neumann).  Each grid point executes the six rules in the reference's order
// (x-low, x-high, y-low, y-high, z-low, z-high); reads use the pre-launch
// snapshot (see header).
void orc_SetFaceBCs(double* X_, const int* type6, const double* val6, i64 nx, i64 ny, i64 nz) {
    const i64 n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    std::vector<double> snap(X_, X_ + n1 * n2 * n3);
    A3 X = mk(X_, n1, n2, n3), S = mk(snap.data(), n1, n2, n3);
    auto rule = [&](int f, double inner) { return type6[f] == 0 ? inner : 2.0 * val6[f] - inner; };
    PARFOR3(n1, n2, n3) {
        if (i == 0) X(i, j, k) = rule(0, S(1, j, k));
        if (i == n1 - 1) X(i, j, k) = rule(1, S(n1 - 2, j, k));
        if (j == 0) X(i, j, k) = rule(2, S(i, 1, k));
        if (j == n2 - 1) X(i, j, k) = rule(3, S(i, n2 - 2, k));
        if (k == 0) X(i, j, k) = rule(4, S(i, j, 1));
        if (k == n3 - 1) X(i, j, k) = rule(5, S(i, j, n3 - 2));
    }
}

// KillNorthSouthFluxes!  Dimensionless/HydroThermal3D_Alban_v6.jl:153-159
void orc_KillNorthSouthFluxes(double* Ty_, i64 nx, i64 ny, i64 nz) {
    A3 Ty = mk(Ty_, nx, ny + 1, nz);
    PARFOR3(nx, ny + 1, nz) {
        if (j == 0) Ty(i, j, k) = 0.0;
        if (j == ny) Ty(i, j, k) = 0.0;
    }
}

// ResetA!  tools/Macros.jl:171-177 (two arrays of n elements each)
void orc_ResetA(double* A, double* B, i64 n) {
#pragma omp parallel for
    for (i64 t = 0; t < n; ++t) { A[t] = 0.0; B[t] = 0.0; }
}
// Cpy_inn_to_all!  tools/Macros.jl:187-192 : A (n^3) = inn(B (n+2)^3)
void orc_Cpy_inn_to_all(double* A_, const double* B_, i64 nx, i64 ny, i64 nz) {
    A3 A = mk(A_, nx, ny, nz), B = mk((double*)B_, nx + 2, ny + 2, nz + 2);
    PARFOR3(nx, ny, nz) { A(i, j, k) = INN(B); }
}
// Cpy_all_to_inn!  tools/Macros.jl:194-199
void orc_Cpy_all_to_inn(double* A_, const double* B_, i64 nx, i64 ny, i64 nz) {
    A3 A = mk(A_, nx + 2, ny + 2, nz + 2), B = mk((double*)B_, nx, ny, nz);
    PARFOR3(nx, ny, nz) { INN(A) = B(i, j, k); }
}
// ArrayEqualArray!  tools/Weno5_Routines.jl:271-276
void orc_ArrayEqualArray(double* A, const double* B, i64 n) {
#pragma omp parallel for
    for (i64 t = 0; t < n; ++t) A[t] = B[t];
}
// Multiply  Dimensional/kernels_HT3D_dimensional.jl:106-109
void orc_Multiply(double* a, const double* b, const double* c, i64 n) {
#pragma omp parallel for
    for (i64 t = 0; t < n; ++t) a[t] = b[t] * c[t];
}

// ===========================================================================
// Reductions  (tools/Macros.jl:20-25: maximum_g, minimum_g, mean_g, sum_g).
// Sequential in index order so the oracle is reproducible.
// ===========================================================================
double orc_sum(const double* a, i64 n) { double s = 0.0; for (i64 t = 0; t < n; ++t) s += a[t]; return s; }
double orc_sum_abs(const double* a, i64 n) { double s = 0.0; for (i64 t = 0; t < n; ++t) s += std::fabs(a[t]); return s; }
double orc_max(const double* a, i64 n) { double m = -INFINITY; for (i64 t = 0; t < n; ++t) m = std::max(m, a[t]); return m; }
double orc_min(const double* a, i64 n) { double m = INFINITY; for (i64 t = 0; t < n; ++t) m = std::min(m, a[t]); return m; }
double orc_max_abs(const double* a, i64 n) { double m = 0.0; for (i64 t = 0; t < n; ++t) m = std::max(m, std::fabs(a[t])); return m; }

// ===========================================================================
// WENO5 v1 (tools/Weno5_Routines.jl) -- unfused, as the dimensionless
// drivers call it.
// ===========================================================================

// V{x,y,z}PlusMinus!  tools/Weno5_Routines.jl:5-42.  Vm/Vp are n^3.
void orc_VPlusMinus(double* Vm_, double* Vp_, const double* V_, int axis, i64 nx, i64 ny, i64 nz) {
    A3 Vm = mk(Vm_, nx, ny, nz), Vp = mk(Vp_, nx, ny, nz);
    A3 V = mk((double*)V_, nx + (axis == 0), ny + (axis == 1), nz + (axis == 2));
    const i64 di = axis == 0, dj = axis == 1, dk = axis == 2;
    PARFOR3(nx, ny, nz) {
        const double a = V(i, j, k), b = V(i + di, j + dj, k + dk);
        if (a < 0.0) Vm(i, j, k) = a;
        if (a > 0.0) Vm(i, j, k) = 0.0;
        if (b < 0.0) Vp(i, j, k) = 0.0;
        if (b > 0.0) Vp(i, j, k) = b;
    }
}

// dFdx_Weno5! body (tools/Weno5_Routines.jl:44-68, also inlined in
// tools/Weno5_Routines_v2.jl:70-85).
static inline double weno5_flux(double v1, double v2, double v3, double v4, double v5) {
    const double p1 = v1 / 3.0 - 7.0 / 6.0 * v2 + 11.0 / 6.0 * v3;
    const double p2 = -v2 / 6.0 + 5.0 / 6.0 * v3 + v4 / 3.0;
    const double p3 = v3 / 3.0 + 5.0 / 6.0 * v4 - v5 / 6.0;
    const double maxV = std::max(std::max(std::max(std::max(v1 * v1, v2 * v2), v3 * v3), v4 * v4), v5 * v5);
    const double e = 1e-99 + 1e-6 * maxV;
    double w1 = 13.0 / 12.0 * ((v1 - 2.0 * v2 + v3) * (v1 - 2.0 * v2 + v3)) + 1.0 / 4.0 * ((v1 - 4.0 * v2 + 3.0 * v3) * (v1 - 4.0 * v2 + 3.0 * v3));
    double w2 = 13.0 / 12.0 * ((v2 - 2.0 * v3 + v4) * (v2 - 2.0 * v3 + v4)) + 1.0 / 4.0 * ((v2 - v4) * (v2 - v4));
    double w3 = 13.0 / 12.0 * ((v3 - 2.0 * v4 + v5) * (v3 - 2.0 * v4 + v5)) + 1.0 / 4.0 * ((3.0 * v3 - 4.0 * v4 + v5) * (3.0 * v3 - 4.0 * v4 + v5));
    w1 = 0.1 / ((w1 + e) * (w1 + e));
    w2 = 0.6 / ((w2 + e) * (w2 + e));
    w3 = 0.3 / ((w3 + e) * (w3 + e));
    const double w = (w1 + w2 + w3);
    w1 = w1 / w; w2 = w2 / w; w3 = w3 / w;
    return w1 * p1 + w2 * p2 + w3 * p3;
}

void orc_dFdx_Weno5(double* dF, const double* v1, const double* v2, const double* v3, const double* v4, const double* v5, i64 n) {
#pragma omp parallel for
    for (i64 t = 0; t < n; ++t) dF[t] = weno5_flux(v1[t], v2[t], v3[t], v4[t], v5[t]);
}

// Gradients_{minus,plus}_{x,y,z}_Weno5!  tools/Weno5_Routines.jl:70-128.
// sign = -1 (minus) or +1 (plus); exxx is (n+6)^3; v* are n^3.
void orc_Gradients_Weno5(double* v1_, double* v2_, double* v3_, double* v4_, double* v5_, const double* X_,
                         int axis, int sign, double _dx, double _dy, double _dz, i64 nx, i64 ny, i64 nz) {
    A3 X = mk((double*)X_, nx + 6, ny + 6, nz + 6);
    double* vv[5] = {v1_, v2_, v3_, v4_, v5_};
    const i64 di = axis == 0, dj = axis == 1, dk = axis == 2;
    const double h = axis == 0 ? _dx : (axis == 1 ? _dy : _dz);
    PARFOR3(nx, ny, nz) {
        const i64 I = i + 3, J = j + 3, K = k + 3, c = i + nx * (j + ny * k);
        auto x = [&](int o) { return X(I + o * di, J + o * dj, K + o * dk); };
        if (sign < 0) {
            vv[0][c] = h * (x(-2) - x(-3));
            vv[1][c] = h * (x(-1) - x(-2));
            vv[2][c] = h * (x(0) - x(-1));
            vv[3][c] = h * (x(1) - x(0));
            vv[4][c] = h * (x(2) - x(1));
        } else {
            vv[0][c] = h * (x(3) - x(2));
            vv[1][c] = h * (x(2) - x(1));
            vv[2][c] = h * (x(1) - x(0));
            vv[3][c] = h * (x(0) - x(-1));
            vv[4][c] = h * (x(-1) - x(-2));
        }
    }
}

// Boundaries_{x,y,z}_Weno5!  v1: tools/Weno5_Routines.jl:130-255 (Fc is n^3,
// ex_src = 0); v2: tools/Weno5_Routines_v2.jl:221-347 (Fc is the ghosted
// (n+2)^3 array, ex_src = 1).  type: 0 Neumann, 1 Dirichlet, 2 periodic.
void orc_Boundaries_Weno5(double* X_, const double* Fc_, int axis, int typeL, double valL, int typeR, double valR,
                          int ex_src, i64 nx, i64 ny, i64 nz) {
    const i64 o = ex_src ? 1 : 0;
    A3 X = mk(X_, nx + 6, ny + 6, nz + 6), F = mk((double*)Fc_, nx + 2 * o, ny + 2 * o, nz + 2 * o);
    const i64 N[3] = {nx, ny, nz};
    PARFOR3(nx + 6, ny + 6, nz + 6) {
        if (i < nx && j < ny && k < nz) X(i + 3, j + 3, k + 3) = F(i + o, j + o, k + o);
        const i64 idx[3] = {i, j, k};
        // the two axes other than `axis` must be inner (3 <= . < N+3)
        bool lateral = true;
        for (int a = 0; a < 3; ++a)
            if (a != axis && !(idx[a] >= 3 && idx[a] < N[a] + 3)) lateral = false;
        if (!lateral) continue;
        const i64 p = idx[axis], n = N[axis];
        auto src = [&](i64 m) {  // inner index m along axis, others from position
            i64 s[3] = {i - 3, j - 3, k - 3};
            s[axis] = m;
            return F(s[0] + o, s[1] + o, s[2] + o);
        };
        if (p < 3) {
            const i64 m = 2 - p;  // p=0 -> 2, 1 -> 1, 2 -> 0
            if (typeL == 0) X(i, j, k) = src(m);
            if (typeL == 1) X(i, j, k) = 2 * valL - src(m);
            if (typeL == 2) X(i, j, k) = src(n - 3 + p);
        } else if (p >= n + 3) {
            const i64 q = p - (n + 3);     // 0,1,2
            const i64 m = n - 1 - q;       // mirror
            if (typeR == 0) X(i, j, k) = src(m);
            if (typeR == 1) X(i, j, k) = 2 * valR - src(m);
            if (typeR == 2) X(i, j, k) = src(q);
        }
    }
}

// Advect!  v1  tools/Weno5_Routines.jl:257-262
void orc_Advect_v1(double* Fc, const double* Vxp, const double* dTdxm, const double* Vxm, const double* dTdxp, double dt, i64 n) {
#pragma omp parallel for
    for (i64 t = 0; t < n; ++t) Fc[t] = Fc[t] - dt * (Vxp[t] * dTdxm[t] + Vxm[t] * dTdxp[t]);
}
// TimeAveraging!  v1  tools/Weno5_Routines.jl:264-269
void orc_TimeAveraging_v1(double* Fc, const double* Fold, double order, i64 n) {
#pragma omp parallel for
    for (i64 t = 0; t < n; ++t) Fc[t] = (1.0 / order) * Fc[t] + (1.0 - 1.0 / order) * Fold[t];
}

// AdvectWithWeno5 (v1 orchestration)  Dimensionless/kernels_HT3D.jl:156-233
// without the Init_vel! call at its top (the caller computes V first).
// Temporaries are allocated here.  bc_type[6]/bc_val[6]: W,E,S,N,B,F.
void orc_AdvectWithWeno5_v1(double* Tc_ex, const double* Vx, const double* Vy, const double* Vz, double dt,
                            double _dx, double _dy, double _dz, const int* bc_type, const double* bc_val,
                            i64 nx, i64 ny, i64 nz) {
    const i64 n = nx * ny * nz, nxxx = (nx + 6) * (ny + 6) * (nz + 6);
    std::vector<double> Tc(n), Told(n), exxx(nxxx, 0.0), v[5], dm(n), dp(n), Vm[3], Vp[3];
    for (auto& a : v) a.assign(n, 0.0);
    const double* V[3] = {Vx, Vy, Vz};
    for (int a = 0; a < 3; ++a) {
        Vm[a].assign(n, 0.0); Vp[a].assign(n, 0.0);  // ResetA!
        orc_VPlusMinus(Vm[a].data(), Vp[a].data(), V[a], a, nx, ny, nz);
    }
    orc_Cpy_inn_to_all(Tc.data(), Tc_ex, nx, ny, nz);
    const double order = 2.0;
    for (int a = 0; a < 3; ++a) {
        orc_ArrayEqualArray(Told.data(), Tc.data(), n);
        for (int io = 1; io <= (int)order; ++io) {
            orc_Boundaries_Weno5(exxx.data(), Tc.data(), a, bc_type[2 * a], bc_val[2 * a], bc_type[2 * a + 1],
                                 bc_val[2 * a + 1], 0, nx, ny, nz);
            orc_Gradients_Weno5(v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(), exxx.data(), a, -1,
                                _dx, _dy, _dz, nx, ny, nz);
            orc_dFdx_Weno5(dm.data(), v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(), n);
            orc_Gradients_Weno5(v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(), exxx.data(), a, +1,
                                _dx, _dy, _dz, nx, ny, nz);
            orc_dFdx_Weno5(dp.data(), v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data(), n);
            orc_Advect_v1(Tc.data(), Vp[a].data(), dm.data(), Vm[a].data(), dp.data(), dt, n);
        }
        orc_TimeAveraging_v1(Tc.data(), Told.data(), order, n);
    }
    orc_Cpy_all_to_inn(Tc_ex, Tc.data(), nx, ny, nz);
}

// ===========================================================================
// WENO5 v2 (tools/Weno5_Routines_v2.jl) -- fused per-axis Advect!.
// quirk = 1 reproduces the reference's minus-branch stencil
// v5 = (X[I+2]-X[I-1])/dx (tools/Weno5_Routines_v2.jl:69,119,169);
// quirk = 0 uses the textbook X[I+2]-X[I+1] (as in tools/Weno5_Routines.jl:76).
// ===========================================================================
void orc_Advect_v2(double* Fc_, const double* X_, const double* V_, int axis, double dt, double _dx, double _dy,
                   double _dz, int quirk, i64 nx, i64 ny, i64 nz) {
    A3 Fc = mk(Fc_, nx + 2, ny + 2, nz + 2), X = mk((double*)X_, nx + 6, ny + 6, nz + 6);
    A3 V = mk((double*)V_, nx + (axis == 0), ny + (axis == 1), nz + (axis == 2));
    const i64 di = axis == 0, dj = axis == 1, dk = axis == 2;
    const double h = axis == 0 ? _dx : (axis == 1 ? _dy : _dz);
    PARFOR3(nx, ny, nz) {
        const i64 I = i + 3, J = j + 3, K = k + 3;
        auto x = [&](int o) { return X(I + o * di, J + o * dj, K + o * dk); };
        const double a = V(i, j, k), b = V(i + di, j + dj, k + dk);
        double Vm = 0.0, Vp = 0.0;
        if (a < 0.0) Vm = a;
        if (a >= 0.0) Vm = 0.0;
        if (b < 0.0) Vp = 0.0;
        if (b >= 0.0) Vp = b;
        const double m1 = h * (x(-2) - x(-3)), m2 = h * (x(-1) - x(-2)), m3 = h * (x(0) - x(-1)), m4 = h * (x(1) - x(0));
        const double m5 = quirk ? h * (x(2) - x(-1)) : h * (x(2) - x(1));
        const double dFdxm = weno5_flux(m1, m2, m3, m4, m5);
        const double p1 = h * (x(3) - x(2)), p2 = h * (x(2) - x(1)), p3 = h * (x(1) - x(0)), p4 = h * (x(0) - x(-1));
        const double p5 = h * (x(-1) - x(-2));
        const double dFdxp = weno5_flux(p1, p2, p3, p4, p5);
        Fc(i + 1, j + 1, k + 1) = Fc(i + 1, j + 1, k + 1) - dt * (Vp * dFdxm + Vm * dFdxp);
    }
}
// TimeAveraging!  v2  tools/Weno5_Routines_v2.jl:214-219 (Fold is n^3)
void orc_TimeAveraging_v2(double* Fc_, const double* Fold_, double order, i64 nx, i64 ny, i64 nz) {
    A3 Fc = mk(Fc_, nx + 2, ny + 2, nz + 2), Fold = mk((double*)Fold_, nx, ny, nz);
    PARFOR3(nx, ny, nz) { INN(Fc) = (1.0 / order) * INN(Fc) + (1.0 - 1.0 / order) * Fold(i, j, k); }
}
// AdvectWithWeno5_v2  tools/Weno5_Routines_v2.jl:1-50
void orc_AdvectWithWeno5_v2(double* Tc_ex, const double* Vx, const double* Vy, const double* Vz, double dt,
                            double _dx, double _dy, double _dz, const int* bc_type, const double* bc_val, int quirk,
                            i64 nx, i64 ny, i64 nz) {
    const i64 n = nx * ny * nz, nxxx = (nx + 6) * (ny + 6) * (nz + 6);
    std::vector<double> Told(n), exxx(nxxx, 0.0);
    const double* V[3] = {Vx, Vy, Vz};
    const double order = 2.0;
    for (int a = 0; a < 3; ++a) {
        orc_Cpy_inn_to_all(Told.data(), Tc_ex, nx, ny, nz);
        for (int io = 1; io <= (int)order; ++io) {
            orc_Boundaries_Weno5(exxx.data(), Tc_ex, a, bc_type[2 * a], bc_val[2 * a], bc_type[2 * a + 1],
                                 bc_val[2 * a + 1], 1, nx, ny, nz);
            orc_Advect_v2(Tc_ex, exxx.data(), V[a], a, dt, _dx, _dy, _dz, quirk, nx, ny, nz);
        }
        orc_TimeAveraging_v2(Tc_ex, Told.data(), order, nx, ny, nz);
    }
}

// ===========================================================================
// Dimensional kernels  (Dimensional/kernels_HT3D_dimensional.jl) and the
// material laws of Dimensional/HydroThermal3D_v18.jl:29-39.
// ===========================================================================
static inline double kTs(double T) { return 3.1138 - 0.0023 * (T); }
static inline double kTf(double T) { return -0.069 + 0.0012 * (T); }
static inline double Cf(double T) { return 1000 + 7.5 * (T); }
static inline double Cs(double T) { return 0.5915 * (T) + 636.14; }
static inline double rho_s(double T) { return 2800 * (1 - (0.000024 * (T - 293))); }
static inline double rhof_C(double T_C, double p) {
    const double p2 = p * p, p3 = p * p * p, p4 = p2 * p2, T2 = T_C * T_C, T3 = T_C * T_C * T_C, T4 = T2 * T2;
    return 1006 + (7.424e-7 * p) + (-0.3922 * T_C) + (-4.441e-15 * p2) + (4.547e-9 * p * T_C) + (-0.003774 * T2) +
           (1.451e-23 * p3) + (-1.793e-17 * p2 * T_C) + (7.485e-12 * p * T2) + (2.955e-6 * T3) + (-1.463e-32 * p4) +
           (1.361e-26 * p3 * T_C) + (4.018e-21 * (p2) * (T2)) + (-7.372e-15 * p * T3) + (5.698e-11 * T4);
}
static inline double drhodP_C(double T_C, double p) {
    const double T2 = T_C * T_C, T3 = T_C * T_C * T_C, p2 = p * p, p3 = p * p * p;
    return -7.372e-15 * T3 + 8.036e-21 * T2 * p + 7.485e-12 * T2 + 4.083e-26 * T_C * p2 - 3.586e-17 * T_C * p +
           4.547e-9 * T_C - 5.852e-32 * p3 + 4.353e-23 * p2 - 8.882e-15 * p + 7.424e-7;
}
// 10^x and e^x: the library's own exponentials (expo.h), so the oracle and the
// device evaluate the laws to the same bits; expo.h is pinned against 40-digit
// decimal arithmetic (below 1 ulp) by the CPU tests.  Julia evaluates
// 10^x with pow and e^x with its own table method, both also below 1 ulp.
static inline double mu_f(double T) { return 2.414e-5 * ht3d_exp10(247.8 / (T - 140.)); }
static inline double k_F(double y, double delta) { return 5e-16 * ht3d_exp(y / delta); }
static inline double phi_of(double phase, double phi0) { return phase == 2.0 ? 3 * phi0 : phi0; }

double orc_law(int which, double a, double b) {
    switch (which) {
        case 0: return kTs(a);
        case 1: return kTf(a);
        case 2: return Cf(a);
        case 3: return Cs(a);
        case 4: return rho_s(a);
        case 5: return rhof_C(a, b);
        case 6: return drhodP_C(a, b);
        case 7: return mu_f(a);
        case 8: return k_F(a, b);
        case 9: return phi_of(a, b);
        case 10: return ht3d_exp(a);
        case 11: return ht3d_exp10(a);
    }
    return NAN;
}

// 8-point vertex average of an extended centre field (Dimensional/kernels_HT3D_dimensional.jl:43-44)
#define VTX8(A) (1.0 / 8.0 * (A(i + 1, j + 1, k + 1) + A(i + 1, j, k + 1) + A(i, j + 1, k + 1) + A(i, j, k + 1)) + \
                 1.0 / 8.0 * (A(i + 1, j + 1, k + 0) + A(i + 1, j, k + 0) + A(i, j + 1, k + 0) + A(i, j, k + 0)))

// ComputeThermalConductivity  :40-50
void orc_ComputeThermalConductivity(double* ktv_, const double* Tce_, const double* phv_, double phi0, double scale_kt,
                                    double scale_T, i64 nx, i64 ny, i64 nz) {
    A3 ktv = mk(ktv_, nx + 1, ny + 1, nz + 1), Tce = mk((double*)Tce_, nx + 2, ny + 2, nz + 2), phv = mk((double*)phv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        double Tv = 1.0 / 8.0 * (Tce(i + 1, j + 1, k + 1) + Tce(i + 1, j, k + 1) + Tce(i, j + 1, k + 1) + Tce(i, j, k + 1));
        Tv += 1.0 / 8.0 * (Tce(i + 1, j + 1, k + 0) + Tce(i + 1, j, k + 0) + Tce(i, j + 1, k + 0) + Tce(i, j, k + 0));
        Tv *= scale_T;
        const double ph = phv(i, j, k);
        ktv(i, j, k) = ((1 - phi_of(ph, phi0)) * kTs(Tv) + phi_of(ph, phi0) * kTf(Tv)) / scale_kt;
    }
}

// ComputeHydroConductivity  :52-86.  kmul_v (optional, may be NULL) is a
// vertex multiplier of the permeability law kF(y) used for heterogeneous
// permeability fields; NULL reproduces the reference exactly.
void orc_ComputeHydroConductivity(double* kfv_, const double* Tce_, const double* Pce_, const double* phv_, double ymin,
                                  double dy, double k_fact, double delta, double scale_s, double scale_T, double scale_L,
                                  double scale_t, double scale_eta, int mode, const double* kmul_v,
                                  i64 nx, i64 ny, i64 nz) {
    A3 kfv = mk(kfv_, nx + 1, ny + 1, nz + 1), Tce = mk((double*)Tce_, nx + 2, ny + 2, nz + 2), Pce = mk((double*)Pce_, nx + 2, ny + 2, nz + 2);
    A3 phv = mk((double*)phv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        double Tv = 1.0 / 8.0 * (Tce(i + 1, j + 1, k + 1) + Tce(i + 1, j, k + 1) + Tce(i, j + 1, k + 1) + Tce(i, j, k + 1));
        Tv += 1.0 / 8.0 * (Tce(i + 1, j + 1, k + 0) + Tce(i + 1, j, k + 0) + Tce(i, j + 1, k + 0) + Tce(i, j, k + 0));
        Tv *= scale_T;
        if (Tv < 293.15) Tv = 293.15;
        double Pv = 1.0 / 8.0 * (Pce(i + 1, j + 1, k + 1) + Pce(i + 1, j, k + 1) + Pce(i, j + 1, k + 1) + Pce(i, j, k + 1));
        Pv += 1.0 / 8.0 * (Pce(i + 1, j + 1, k + 0) + Pce(i + 1, j, k + 0) + Pce(i, j + 1, k + 0) + Pce(i, j, k + 0));
        Pv *= scale_s;
        const double y = ymin + (double)j * dy;
        double kF = k_F(y * scale_L, delta * scale_L);
        if (kmul_v) kF *= kmul_v[i + (nx + 1) * (j + (ny + 1) * k)];
        const double rk_mu = rhof_C(Tv - 273.15, Pv) * kF / mu_f(Tv);
        if (mode == 1) kfv(i, j, k) = rk_mu / scale_t;
        else if (mode == 2) kfv(i, j, k) = (kF / mu_f(Tv)) / (scale_L * scale_L / scale_eta);
        else if (mode == 3) kfv(i, j, k) = kF / (scale_L * scale_L);
        if (phv(i, j, k) == 2.0) kfv(i, j, k) *= k_fact;
    }
}

// ComputeFluidDensity  :88-104
void orc_ComputeFluidDensity(double* rfv_, const double* Tce_, const double* Pce_, const double* phv_, double scale_s,
                             double scale_T, double scale_rho, i64 nx, i64 ny, i64 nz) {
    A3 rfv = mk(rfv_, nx + 1, ny + 1, nz + 1), Tce = mk((double*)Tce_, nx + 2, ny + 2, nz + 2), Pce = mk((double*)Pce_, nx + 2, ny + 2, nz + 2);
    A3 phv = mk((double*)phv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        double Tv = 1.0 / 8.0 * (Tce(i + 1, j + 1, k + 1) + Tce(i + 1, j, k + 1) + Tce(i, j + 1, k + 1) + Tce(i, j, k + 1));
        Tv += 1.0 / 8.0 * (Tce(i + 1, j + 1, k + 0) + Tce(i + 1, j, k + 0) + Tce(i, j + 1, k + 0) + Tce(i, j, k + 0));
        Tv *= scale_T;
        double Pv = 1.0 / 8.0 * (Pce(i + 1, j + 1, k + 1) + Pce(i + 1, j, k + 1) + Pce(i, j + 1, k + 1) + Pce(i, j, k + 1));
        Pv += 1.0 / 8.0 * (Pce(i + 1, j + 1, k + 0) + Pce(i + 1, j, k + 0) + Pce(i, j + 1, k + 0) + Pce(i, j, k + 0));
        Pv *= scale_s;
        rfv(i, j, k) = rhof_C(Tv - 273.15, Pv) / scale_rho;
        if (phv(i, j, k) == 1.0) rfv(i, j, k) = 0.000 / scale_rho;
    }
}

// SmoothConductivityV2C  :111-114  (ktc n^3 <- av(ktv))
void orc_SmoothConductivityV2C(double* ktc_, const double* ktv_, i64 nx, i64 ny, i64 nz) {
    A3 ktc = mk(ktc_, nx, ny, nz), ktv = mk((double*)ktv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx, ny, nz) { ktc(i, j, k) = AV(ktv); }
}
// SmoothConductivityC2V  :116-119  (inn(ktv) <- av(ktc)), range (n-1)^3
void orc_SmoothConductivityC2V(double* ktv_, const double* ktc_, i64 nx, i64 ny, i64 nz) {
    A3 ktv = mk(ktv_, nx + 1, ny + 1, nz + 1), ktc = mk((double*)ktc_, nx, ny, nz);
    PARFOR3(nx - 1, ny - 1, nz - 1) { INN(ktv) = AV(ktc); }
}
// SwapDYREL!  :122-126
void orc_SwapDYREL(double* Xc_, double* Yc, const double* X0c_ex_, const double* Y0c, i64 nx, i64 ny, i64 nz) {
    A3 Xc = mk(Xc_, nx, ny, nz), X0 = mk((double*)X0c_ex_, nx + 2, ny + 2, nz + 2);
    PARFOR3(nx, ny, nz) {
        Xc(i, j, k) = INN(X0);
        const i64 c = i + nx * (j + ny * k);
        Yc[c] = Y0c[c];
    }
}
// InitThermal! (dimensional)  :128-131  Tc0 <- inn(Tc_ex)  (== Cpy_inn_to_all!)
void orc_InitThermal_dim(double* Tc0, const double* Tc_ex, i64 nx, i64 ny, i64 nz) { orc_Cpy_inn_to_all(Tc0, Tc_ex, nx, ny, nz); }
// InitConductivity!  :133-138
void orc_InitConductivity(double* kx_, double* ky_, double* kz_, const double* ktv_, i64 nx, i64 ny, i64 nz) {
    A3 kx = mk(kx_, nx + 1, ny, nz), ky = mk(ky_, nx, ny + 1, nz), kz = mk(kz_, nx, ny, nz + 1), kv = mk((double*)ktv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        if (i < nx + 1 && j < ny && k < nz) kx(i, j, k) = AV_YZA(kv);
        if (i < nx && j < ny + 1 && k < nz) ky(i, j, k) = AV_XZA(kv);
        if (i < nx && j < ny && k < nz + 1) kz(i, j, k) = AV_XYA(kv);
    }
}
// ComputeρCeffective!  :148-160
void orc_ComputeRhoCeffective(double* rC_, const double* Tc_ex_, const double* Pc_ex_, const double* phc_ex_, double phii,
                              double sca_T, double sca_s, double sca_C, double sca_rho, i64 nx, i64 ny, i64 nz) {
    A3 rC = mk(rC_, nx, ny, nz), T = mk((double*)Tc_ex_, nx + 2, ny + 2, nz + 2), P = mk((double*)Pc_ex_, nx + 2, ny + 2, nz + 2);
    A3 ph_ = mk((double*)phc_ex_, nx + 2, ny + 2, nz + 2);
    PARFOR3(nx, ny, nz) {
        const double ph = INN(ph_);
        if (std::fabs(ph) != 1.0) {
            const double Tsca = INN(T) * sca_T, Psca = INN(P) * sca_s;
            const double r_eff = phi_of(ph, phii) * rhof_C(Tsca - 273.15, Psca) + (1.0 - phi_of(ph, phii)) * rho_s(Tsca);
            const double Ceff = phi_of(ph, phii) * Cf(Tsca) + (1.0 - phi_of(ph, phii)) * Cs(Tsca);
            rC(i, j, k) = (r_eff * Ceff) / sca_rho / sca_C;
        }
    }
}
// ResidualTemperatureLinearised!  :162-181
void orc_ResidualTemperatureLinearised(double* F_, const double* Tc_ex_, const double* Tc_old_, const double* rC_,
                                       const double* phc_ex_, const double* PC_, const double* qx_, const double* qy_,
                                       const double* qz_, double Qt, double transient, double _dt, double _dx,
                                       double _dy, double _dz, i64 nx, i64 ny, i64 nz) {
    A3 F = mk(F_, nx, ny, nz), T = mk((double*)Tc_ex_, nx + 2, ny + 2, nz + 2), T0 = mk((double*)Tc_old_, nx, ny, nz);
    A3 rC = mk((double*)rC_, nx, ny, nz), ph_ = mk((double*)phc_ex_, nx + 2, ny + 2, nz + 2), PC = mk((double*)PC_, nx, ny, nz);
    A3 qx = mk((double*)qx_, nx + 1, ny, nz), qy = mk((double*)qy_, nx, ny + 1, nz), qz = mk((double*)qz_, nx, ny, nz + 1);
    PARFOR3(nx, ny, nz) {
        const double ph = INN(ph_);
        if (std::fabs(ph) != 1.0) {
            double Q = 0.;
            if (ph == 3.0) Q = Qt;
            double f = transient * rC(i, j, k) * _dt * (INN(T) - T0(i, j, k));
            f += (qx(i + 1, j, k) - qx(i, j, k)) * _dx;
            f += (qy(i, j + 1, k) - qy(i, j, k)) * _dy;
            f += (qz(i, j, k + 1) - qz(i, j, k)) * _dz;
            f -= transient * Q;
            f /= PC(i, j, k);
            F(i, j, k) = f;
        } else {
            F(i, j, k) = 0.;
        }
    }
}
// SetTemperatureBCs! (dimensional)  :183-205 (snapshot semantics, see header)
void orc_SetTemperatureBCs_dim(double* T_, const double* ky_, const double* wN_, const double* phc_ex_, double qyS,
                               double _dy, double TN, i64 nx, i64 ny, i64 nz) {
    const i64 n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    std::vector<double> snap(T_, T_ + n1 * n2 * n3);
    A3 T = mk(T_, n1, n2, n3), S = mk(snap.data(), n1, n2, n3), ph = mk((double*)phc_ex_, n1, n2, n3);
    A3 ky = mk((double*)ky_, nx, ny + 1, nz);
    A2 wN{(double*)wN_, nx + 2, nz + 2};
    PARFOR3(n1, n2, n3) {
        if (ph(i, j, k) == 1.0) T(i, j, k) = TN;
        if (i == 0 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= n3 - 1) T(i, j, k) = S(1, j, k);
        if (i == n1 - 1 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= n3 - 1) T(i, j, k) = S(n1 - 2, j, k);
        if (j == 0 && i >= 1 && i <= n1 - 2 && k >= 1 && k <= n3 - 2) {
            const double kS = ky(i - 1, 0, k - 1);
            T(i, j, k) = qyS / _dy / kS + S(i, 1, k);
        }
        if (ph(i, j, k) == -1.0 && j >= 1) T(i, j, k) = (TN - (1.0 - wN(i, k)) * S(i, j - 1, k)) / wN(i, k);
        if (k == 0 && i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2) T(i, j, k) = S(i, j, 1);
        if (k == n3 - 1 && i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2) T(i, j, k) = S(i, j, n3 - 2);
    }
}
// GershgorinPoisson!  :207-221  (expression from notebooks/Gershgorin_TH3D.ipynb cell 2)
void orc_GershgorinPoisson(double* G_, double* D_, const double* rC_, const double* kx_, const double* ky_,
                           const double* kz_, double transient, double dt, double dx, double dy, double dz,
                           i64 nx, i64 ny, i64 nz) {
    A3 G = mk(G_, nx, ny, nz), D = mk(D_, nx, ny, nz), rC = mk((double*)rC_, nx, ny, nz);
    A3 kx = mk((double*)kx_, nx + 1, ny, nz), ky = mk((double*)ky_, nx, ny + 1, nz), kz = mk((double*)kz_, nx, ny, nz + 1);
    PARFOR3(nx, ny, nz) {
        const double kW = kx(i, j, k), kE = kx(i + 1, j, k), kS = ky(i, j, k), kN = ky(i, j + 1, k), kF = kz(i, j, k + 1),
                     kB = kz(i, j, k), rhoC = rC(i, j, k);
        const double diag = ((kB / dz + kF / dz) / dz + (kN / dy + kS / dy) / dy + (kE / dx + kW / dx) / dx + rhoC * transient / dt);
        double g = std::fabs(kE / (dx * dx)) + std::fabs(kW / (dx * dx)) + std::fabs(kN / (dy * dy)) + std::fabs(kS / (dy * dy)) +
                   std::fabs(kB / (dz * dz)) + std::fabs(kF / (dz * dz)) + std::fabs(diag);
        D(i, j, k) = diag;
        g /= diag;
        G(i, j, k) = g;
    }
}
// ϕρf  :225-235 ; ϕρf_old :237-247 (cell inputs) ; ϕdρdP! :249-259
void orc_phi_rhof(double* out_, const double* T_, const double* P_, const double* phc_ex_, double phii, double scale_rho,
                  double scale_T, double scale_s, int cell_inputs, int deriv, i64 nx, i64 ny, i64 nz) {
    A3 out = mk(out_, nx, ny, nz), ph_ = mk((double*)phc_ex_, nx + 2, ny + 2, nz + 2);
    const i64 o = cell_inputs ? 0 : 1;
    A3 T = mk((double*)T_, nx + 2 * o, ny + 2 * o, nz + 2 * o), P = mk((double*)P_, nx + 2 * o, ny + 2 * o, nz + 2 * o);
    PARFOR3(nx, ny, nz) {
        const double ph = INN(ph_);
        if (ph != 1.0) {
            const double Tc = T(i + o, j + o, k + o) * scale_T - 273.15;
            const double Pc = P(i + o, j + o, k + o) * scale_s;
            if (deriv) out(i, j, k) = phi_of(ph, phii) * drhodP_C(Tc, Pc) / (scale_rho / scale_s);
            else out(i, j, k) = phi_of(ph, phii) * rhof_C(Tc, Pc) / scale_rho;
        }
    }
}
// ComputeDarcyFlux!  :266-272
void orc_ComputeDarcyFlux(double* qx_, double* qy_, double* qz_, const double* rfv_, const double* kx_, const double* ky_,
                          const double* kz_, const double* Pf_, double g, double _dx, double _dy, double _dz,
                          i64 nx, i64 ny, i64 nz) {
    A3 qx = mk(qx_, nx + 1, ny, nz), qy = mk(qy_, nx, ny + 1, nz), qz = mk(qz_, nx, ny, nz + 1);
    A3 kx = mk((double*)kx_, nx + 1, ny, nz), ky = mk((double*)ky_, nx, ny + 1, nz), kz = mk((double*)kz_, nx, ny, nz + 1);
    A3 P = mk((double*)Pf_, nx + 2, ny + 2, nz + 2), rfv = mk((double*)rfv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        if (i < nx + 1 && j < ny && k < nz) qx(i, j, k) = -kx(i, j, k) * (_dx * D_XI(P));
        if (i < nx && j < ny + 1 && k < nz) qy(i, j, k) = -ky(i, j, k) * (_dy * D_YI(P) - g * AV_XZA(rfv));
        if (i < nx && j < ny && k < nz + 1) qz(i, j, k) = -kz(i, j, k) * (_dz * D_ZI(P));
    }
}
// ResidualFluidPressure!  :274-289
void orc_ResidualFluidPressure(double* F_, const double* phc_ex_, const double* prf_, const double* prf0_, const double* PC_,
                               const double* qx_, const double* qy_, const double* qz_, double transient, double _dt,
                               double _dx, double _dy, double _dz, i64 nx, i64 ny, i64 nz) {
    A3 F = mk(F_, nx, ny, nz), ph_ = mk((double*)phc_ex_, nx + 2, ny + 2, nz + 2);
    A3 prf = mk((double*)prf_, nx, ny, nz), prf0 = mk((double*)prf0_, nx, ny, nz), PC = mk((double*)PC_, nx, ny, nz);
    A3 qx = mk((double*)qx_, nx + 1, ny, nz), qy = mk((double*)qy_, nx, ny + 1, nz), qz = mk((double*)qz_, nx, ny, nz + 1);
    PARFOR3(nx, ny, nz) {
        const double ph = INN(ph_);
        if (std::fabs(ph) != 1.0) {
            double f = transient * _dt * (prf(i, j, k) - prf0(i, j, k));
            f += (qx(i + 1, j, k) - qx(i, j, k)) * _dx;
            f += (qy(i, j + 1, k) - qy(i, j, k)) * _dy;
            f += (qz(i, j, k + 1) - qz(i, j, k)) * _dz;
            f /= PC(i, j, k);
            F(i, j, k) = f;
        } else {
            F(i, j, k) = 0.;
        }
    }
}
// SetPressureBCs! (dimensional)  :291-314
void orc_SetPressureBCs_dim(double* P_, const double* wN_, const double* phc_ex_, double PN, i64 nx, i64 ny, i64 nz) {
    const i64 n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    std::vector<double> snap(P_, P_ + n1 * n2 * n3);
    A3 P = mk(P_, n1, n2, n3), S = mk(snap.data(), n1, n2, n3), ph = mk((double*)phc_ex_, n1, n2, n3);
    A2 wN{(double*)wN_, nx + 2, nz + 2};
    PARFOR3(n1, n2, n3) {
        if (ph(i, j, k) == 1.0) P(i, j, k) = PN;
        if (i == 0 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= n3 - 2) P(i, j, k) = S(1, j, k);
        if (i == n1 - 1 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= n3 - 2) P(i, j, k) = S(n1 - 2, j, k);
        if (j == 0 && i >= 1 && i <= n1 - 2 && k >= 1 && k <= n3 - 2) P(i, j, k) = S(i, 1, k);
        if (ph(i, j, k) == -1.0 && j >= 1) P(i, j, k) = (PN - (1.0 - wN(i, k)) * S(i, j - 1, k)) / wN(i, k);
        if (k == 0 && i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2) P(i, j, k) = S(i, j, 1);
        if (k == n3 - 1 && i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2) P(i, j, k) = S(i, j, n3 - 2);
    }
}
// Init_vel! (dimensional)  :328-333
void orc_Init_vel_dim(double* Vx_, double* Vy_, double* Vz_, const double* qx_, const double* qy_, const double* qz_,
                      const double* rfv_, i64 nx, i64 ny, i64 nz) {
    A3 Vx = mk(Vx_, nx + 1, ny, nz), Vy = mk(Vy_, nx, ny + 1, nz), Vz = mk(Vz_, nx, ny, nz + 1);
    A3 qx = mk((double*)qx_, nx + 1, ny, nz), qy = mk((double*)qy_, nx, ny + 1, nz), qz = mk((double*)qz_, nx, ny, nz + 1);
    A3 rfv = mk((double*)rfv_, nx + 1, ny + 1, nz + 1);
    PARFOR3(nx + 1, ny + 1, nz + 1) {
        if (i < nx + 1 && j < ny && k < nz) Vx(i, j, k) = qx(i, j, k) / AV_YZA(rfv);
        if (i < nx && j < ny + 1 && k < nz) Vy(i, j, k) = qy(i, j, k) / AV_XZA(rfv);
        if (i < nx && j < ny && k < nz + 1) Vz(i, j, k) = qz(i, j, k) / AV_XYA(rfv);
    }
}
// GershgorinHydro!  :335-347
void orc_GershgorinHydro(double* G_, const double* s_, const double* kx_, const double* ky_, const double* kz_,
                         double transient, double dt, double dx, double dy, double dz, i64 nx, i64 ny, i64 nz) {
    A3 G = mk(G_, nx, ny, nz), s = mk((double*)s_, nx, ny, nz);
    A3 kx = mk((double*)kx_, nx + 1, ny, nz), ky = mk((double*)ky_, nx, ny + 1, nz), kz = mk((double*)kz_, nx, ny, nz + 1);
    PARFOR3(nx, ny, nz) {
        const double kW = kx(i, j, k), kE = kx(i + 1, j, k), kS = ky(i, j, k), kN = ky(i, j + 1, k), kF = kz(i, j, k + 1),
                     kB = kz(i, j, k), rhoC = s(i, j, k);
        G(i, j, k) = std::fabs(kE / (dx * dx)) + std::fabs(kW / (dx * dx)) + std::fabs(kN / (dy * dy)) + std::fabs(kS / (dy * dy)) +
                     std::fabs(kB / (dz * dz)) + std::fabs(kF / (dz * dz)) +
                     std::fabs((kB / dz + kF / dz) / dz + (kN / dy + kS / dy) / dy + (kE / dx + kW / dx) / dx + rhoC * transient / dt);
    }
}
// RayleighQuotientNumerator!/Denominator!  :349-363
void orc_RayleighQuotientNumerator(double* G, const double* F0, const double* Fit, const double* F, double dtau, i64 n) {
#pragma omp parallel for
    for (i64 t = 0; t < n; ++t) { const double dx = dtau * F0[t]; G[t] = -dx * (F[t] - Fit[t]); }
}
void orc_RayleighQuotientDenominator(double* G, const double* F0, double dtau, i64 n) {
#pragma omp parallel for
    for (i64 t = 0; t < n; ++t) { const double dx = dtau * F0[t]; G[t] = dx * dx; }
}

}  // extern "C"

// ===========================================================================
// Canonical summation order of the DYREL norm and Rayleigh-quotient sums:
// a 32-ary tree over the linear cell index.  Groups of 32 consecutive values
// are combined by the butterfly-free "shift-down" tree (offsets 16,8,4,2,1:
// v[l] = v[l] + v[l+off] for l < off), 32 group results by the same tree, and
// the resulting per-1024 partials again, level by level, padding with zeros.
// libht3d evaluates its FP64 solver sums in exactly this order (one 1024-
// thread block per group of 1024, warp shuffles), so the plain FP64 solver is
// reproducible bit for bit.
// ===========================================================================
static inline double warp_tree(double* v) {
    for (int off = 16; off > 0; off >>= 1)
        for (int l = 0; l < off; ++l) v[l] = v[l] + v[l + off];
    return v[0];
}
static double tree_sum(const double* a, i64 n) {
    if (n <= 0) return 0.0;
    std::vector<double> cur(a, a + n);
    do {
        const i64 m = ((i64)cur.size() + 1023) / 1024;
        std::vector<double> nxt(m);
#pragma omp parallel for schedule(static)
        for (i64 g = 0; g < m; ++g) {
            double w[32];
            for (int wi = 0; wi < 32; ++wi) {
                double v[32];
                for (int l = 0; l < 32; ++l) {
                    const i64 idx = g * 1024 + wi * 32 + l;
                    v[l] = idx < (i64)cur.size() ? cur[idx] : 0.0;
                }
                w[wi] = warp_tree(v);
            }
            nxt[g] = warp_tree(w);
        }
        cur.swap(nxt);
    } while (cur.size() > 1);
    return cur[0];
}
static double tree_sum_abs(const double* a, i64 n) {
    std::vector<double> b(a, a + n);
    for (auto& x : b) x = std::fabs(x);
    return tree_sum(b.data(), n);
}
extern "C" double orc_tree_sum(const double* a, i64 n) { return tree_sum(a, n); }

// ===========================================================================
// Solver drivers.
// ===========================================================================
extern "C" {

// DYREL parameters / statistics (same field order as ht3d_dyrel_params /
// ht3d_dyrel_stats in include/ht3d.h; the Python harness defines both once).
struct orc_dyrel_params {
    double tol_abs, tol_rel;
    int nitmax, nitout;
    double cfl, cfact, lmin_ratio, norm_scale;
};
struct orc_dyrel_stats {
    int iters, converged, status, checks;
    double nF_abs, nF_rel, nF_ini, lambda_min, lambda_max, h1, h2, dtau;
};
enum { ORC_OK = 0, ORC_ERR_NAN = 3, ORC_ERR_DIVERGED = 4 };

// DYREL solve of a dimensionless diffusion problem:
//   F = (R + cX * X_inn + div q(X)) / PC,  q = -k grad X,
// with face BCs bc_type/bc_val and a Jacobi preconditioner PC from
// GershgorinPoisson! (rhoC = 1, transient = (cX != 0), dt = 1/cX).
// The iteration logic follows Dimensional/HydroThermal3D_v18.jl:432-477
// (parameters :433-439, loop :448-477); the residual is
// ResidualDiffusionTransient! (cX = _dt, Dimensionless/HydroThermal3D_Alban_v6.jl:84-90)
// or ResidualDiffusion! (cX = 0, Dimensionless/kernels_HT3D.jl:128-134),
// divided by PC as in ResidualTemperatureLinearised!.
// F (n^3) and F0 (n^3) are outputs (final residual and DYREL momentum);
// n_iter_fixed > 0 runs exactly that many iterations with no stop test.
int orc_dyrel_solve_dimless(double* X, const double* R, const double* kx, const double* ky, const double* kz,
                            double cX, double dx, double dy, double dz, const int* bc_type, const double* bc_val,
                            const orc_dyrel_params* prm, int n_iter_fixed, double* F, double* F0,
                            orc_dyrel_stats* st, i64 nx, i64 ny, i64 nz) {
    const i64 n = nx * ny * nz;
    const double _dx = 1.0 / dx, _dy = 1.0 / dy, _dz = 1.0 / dz;
    std::vector<double> G(n), PC(n), ones(n, 1.0), Fit(n), dumc(n), qx((nx + 1) * ny * nz), qy(nx * (ny + 1) * nz),
        qz(nx * ny * (nz + 1));
    const double transient = cX != 0.0 ? 1.0 : 0.0, dt = cX != 0.0 ? 1.0 / cX : 1.0;
    orc_GershgorinPoisson(G.data(), PC.data(), ones.data(), kx, ky, kz, transient, dt, dx, dy, dz, nx, ny, nz);
    const double lmax = orc_max(G.data(), n);
    double lmin = lmax / prm->lmin_ratio;
    const double dtau = 2.0 / std::sqrt(lmax) * prm->cfl;
    double c = 2.0 * std::sqrt(lmin) * prm->cfact;
    double h1 = (2 - c * dtau) / (2 + c * dtau), h2 = 2 * dtau / (2 + c * dtau);
    orc_ResetA(F, F0, n);
    double nF_abs = 0., nF_rel = 0., nF_ini = 0.;
    int it_done = 0, converged = 0, status = ORC_OK, checks = 0;
    const int nmax = n_iter_fixed > 0 ? n_iter_fixed : prm->nitmax;
    for (int iter = 1; iter <= nmax; ++iter) {
        const bool check = (iter % prm->nitout == 0) || iter <= 2;
        if (check) std::memcpy(Fit.data(), F, sizeof(double) * n);
        orc_SetFaceBCs(X, bc_type, bc_val, nx, ny, nz);
        orc_ComputeFlux(qx.data(), qy.data(), qz.data(), kx, ky, kz, X, _dx, _dy, _dz, nx, ny, nz);
        if (cX != 0.0)
            orc_ResidualDiffusionTransient(F, X, R, qx.data(), qy.data(), qz.data(), cX, _dx, _dy, _dz, nx, ny, nz);
        else
            orc_ResidualDiffusion(F, R, qx.data(), qy.data(), qz.data(), _dx, _dy, _dz, nx, ny, nz);
#pragma omp parallel for
        for (i64 t = 0; t < n; ++t) F[t] /= PC[t];
        orc_DYRELUpdate(F0, X, F, h1, h2, dtau, nx, ny, nz);
        it_done = iter;
        if (check) {
            ++checks;
            orc_Multiply(dumc.data(), F, PC.data(), n);
            nF_abs = tree_sum_abs(dumc.data(), n) / (double)n / std::sqrt((double)n) * prm->norm_scale;
            if (iter == 1) nF_ini = nF_abs;
            nF_rel = nF_abs / nF_ini;
            if (std::isnan(nF_abs)) { status = ORC_ERR_NAN; break; }
            if (nF_rel > 100) { status = ORC_ERR_DIVERGED; break; }
            if (iter > 1) {
                orc_RayleighQuotientNumerator(dumc.data(), F0, Fit.data(), F, dtau, n);
                lmin = std::fabs(tree_sum(dumc.data(), n));
                orc_RayleighQuotientDenominator(dumc.data(), F0, dtau, n);
                lmin /= std::fabs(tree_sum(dumc.data(), n));
                c = 2.0 * std::sqrt(lmin) * prm->cfact;
                h1 = (2 - c * dtau) / (2 + c * dtau);
                h2 = 2 * dtau / (2 + c * dtau);
            }
            if (n_iter_fixed <= 0 && (nF_abs < prm->tol_abs || nF_rel < prm->tol_rel)) { converged = 1; break; }
        }
    }
    if (st) {
        st->iters = it_done; st->converged = converged; st->status = status; st->checks = checks;
        st->nF_abs = nF_abs; st->nF_rel = nF_rel; st->nF_ini = nF_ini; st->lambda_min = lmin; st->lambda_max = lmax;
        st->h1 = h1; st->h2 = h2; st->dtau = dtau;
    }
    return status;
}

// Time step of the dimensionless Horton-Rogers-Lapwood convection problem,
// composed from the reference's dimensionless kernels with the DYREL solver:
//   thermal  InitThermal! -> DYREL(ResidualDiffusionTransient!/PC)
//            (Dimensionless/HydroThermal3D_Alban_v6.jl:327-342)
//   Darcy    InitDarcy! -> KillNorthSouthFluxes! -> Compute_Rp! ->
//            DYREL(ResidualDiffusion!/PC)  (Alban_v6.jl:353-370)
//   advect   Init_vel! -> AdvectWithWeno5 (v1; Dimensionless/kernels_HT3D.jl:156-233)
//            or AdvectWithWeno5_v2 (tools/Weno5_Routines_v2.jl:1-50)
//   dt       dt_fact/6.1*min(dx,dy,dz)/max|V|  (Dimensionless/HydroThermal3D_v7.jl:220)
struct orc_hrl_params {
    double Ra, dx, dy, dz;
    double dt;                       // in: this step's dt; out: next dt (if dt_adapt)
    double Tbot, Ttop;
    int thermal_bc[6]; double thermal_val[6];
    int darcy_bc[6];   double darcy_val[6];
    int weno_bc[6];    double weno_val[6];
    int weno_variant;                // 0 = v1 (textbook), 1 = v2 with the reference quirk, 2 = v2 textbook
    int kill_ns;                     // apply KillNorthSouthFluxes!
    int dt_adapt;
    int advection;
    double dt_fact;
    orc_dyrel_params thermal, darcy;
    double dt_max;                   // > 0: upper bound of the adapted dt (not in the reference)
};

int orc_step_hrl(double* Tc_ex, double* Pc_ex, const double* ktv, const double* kfv, double* Vx, double* Vy,
                 double* Vz, orc_hrl_params* p, orc_dyrel_stats* st_thermal, orc_dyrel_stats* st_darcy,
                 i64 nx, i64 ny, i64 nz) {
    const i64 n = nx * ny * nz;
    const double _dx = 1.0 / p->dx, _dy = 1.0 / p->dy, _dz = 1.0 / p->dz, _dt = 1.0 / p->dt;
    std::vector<double> R(n), F(n), F0(n), Ty(nx * (ny + 1) * nz), kx((nx + 1) * ny * nz), ky(nx * (ny + 1) * nz),
        kz(nx * ny * (nz + 1));
    // thermal
    orc_InitThermal_dimless(R.data(), kx.data(), ky.data(), kz.data(), Tc_ex, ktv, _dt, nx, ny, nz);
    int s = orc_dyrel_solve_dimless(Tc_ex, R.data(), kx.data(), ky.data(), kz.data(), _dt, p->dx, p->dy, p->dz,
                                    p->thermal_bc, p->thermal_val, &p->thermal, 0, F.data(), F0.data(), st_thermal,
                                    nx, ny, nz);
    if (s) return s;
    // Darcy
    orc_InitDarcy(Ty.data(), kx.data(), ky.data(), kz.data(), Tc_ex, kfv, _dt, nx, ny, nz);
    if (p->kill_ns) orc_KillNorthSouthFluxes(Ty.data(), nx, ny, nz);
    orc_Compute_Rp(R.data(), ky.data(), Ty.data(), p->Ra, _dy, nx, ny, nz);
    s = orc_dyrel_solve_dimless(Pc_ex, R.data(), kx.data(), ky.data(), kz.data(), 0.0, p->dx, p->dy, p->dz,
                                p->darcy_bc, p->darcy_val, &p->darcy, 0, F.data(), F0.data(), st_darcy, nx, ny, nz);
    if (s) return s;
    // velocity + advection
    orc_Init_vel(Vx, Vy, Vz, kx.data(), ky.data(), kz.data(), Pc_ex, Ty.data(), p->Ra, _dx, _dy, _dz, nx, ny, nz);
    if (p->advection) {
        if (p->weno_variant == 0)
            orc_AdvectWithWeno5_v1(Tc_ex, Vx, Vy, Vz, p->dt, _dx, _dy, _dz, p->weno_bc, p->weno_val, nx, ny, nz);
        else
            orc_AdvectWithWeno5_v2(Tc_ex, Vx, Vy, Vz, p->dt, _dx, _dy, _dz, p->weno_bc, p->weno_val,
                                   p->weno_variant == 1, nx, ny, nz);
    }
    if (p->dt_adapt) {
        const double vmax = std::max(std::max(orc_max_abs(Vx, (nx + 1) * ny * nz), orc_max_abs(Vy, nx * (ny + 1) * nz)),
                                     orc_max_abs(Vz, nx * ny * (nz + 1)));
        p->dt = p->dt_fact * 1.0 / 6.1 * std::min(std::min(p->dx, p->dy), p->dz) / vmax;
        if (p->dt_max > 0.0 && p->dt > p->dt_max) p->dt = p->dt_max;
    }
    return ORC_OK;
}

}  // extern "C"

// ===========================================================================
// Dimensional model (Dimensional/HydroThermal3D_v18.jl) -- one time step of
// the driver loop :404-572 with the kernels of
// Dimensional/kernels_HT3D_dimensional.jl and AdvectWithWeno5_v2.
// ===========================================================================
struct orc_v18_params;
extern "C" {
struct orc_v18_params {
    double dx, dy, dz, ymin;
    double dt, time;
    double phi_i, k_fact, delta, g, Qt, qyS;
    double Ttop, Tbot, Ptop, Pbot, T_pluton;
    double C_adv;
    double sc_T, sc_L, sc_t, sc_eta, sc_sigma, sc_rho, sc_C, sc_kt;
    int it, thermal, hydro, advection, dt_constant, weno_variant;
    orc_dyrel_params thermal_dyrel, darcy_dyrel;
    int n_adv;  // out: advection sub-steps taken
    int pad_;
};
}  // extern "C"

// shared DYREL loop for the two dimensional solves; `iteration` performs the
// kernels of one pseudo-iteration (v18:451-455 / :510-514) given h1,h2,dtau.
template <typename IterFn>
static int dyrel_loop(double* X, double* F, double* F0, const double* PC, double lmax, const orc_dyrel_params* prm,
                      IterFn&& iteration, orc_dyrel_stats* st, i64 nx, i64 ny, i64 nz) {
    const i64 n = nx * ny * nz;
    std::vector<double> Xit(n), Fit(n), dumc(n);
    double lmin = lmax / prm->lmin_ratio;
    const double dtau = 2.0 / std::sqrt(lmax) * prm->cfl;
    double c = 2.0 * std::sqrt(lmin) * prm->cfact;
    double h1 = (2 - c * dtau) / (2 + c * dtau), h2 = 2 * dtau / (2 + c * dtau);
    orc_ResetA(F, F0, n);
    double nF_abs = 0., nF_rel = 0., nF_ini = 0.;
    int it_done = 0, converged = 0, status = ORC_OK, checks = 0;
    for (int iter = 1; iter <= prm->nitmax; ++iter) {
        const bool check = (iter % prm->nitout == 0) || iter <= 2;
        if (check) orc_SwapDYREL(Xit.data(), Fit.data(), X, F, nx, ny, nz);
        iteration(h1, h2, dtau);
        it_done = iter;
        if (check) {
            ++checks;
            orc_Multiply(dumc.data(), F, PC, n);
            nF_abs = tree_sum_abs(dumc.data(), n) / (double)n / std::sqrt((double)n) * prm->norm_scale;
            if (iter == 1) nF_ini = nF_abs;
            nF_rel = nF_abs / nF_ini;
            if (std::isnan(nF_abs)) { status = ORC_ERR_NAN; break; }
            if (nF_rel > 100) { status = ORC_ERR_DIVERGED; break; }
            if (iter > 1) {
                orc_RayleighQuotientNumerator(dumc.data(), F0, Fit.data(), F, dtau, n);
                lmin = std::fabs(tree_sum(dumc.data(), n));
                orc_RayleighQuotientDenominator(dumc.data(), F0, dtau, n);
                lmin /= std::fabs(tree_sum(dumc.data(), n));
                c = 2.0 * std::sqrt(lmin) * prm->cfact;
                h1 = (2 - c * dtau) / (2 + c * dtau);
                h2 = 2 * dtau / (2 + c * dtau);
            }
            if (nF_abs < prm->tol_abs || nF_rel < prm->tol_rel) { converged = 1; break; }
        }
    }
    if (st) {
        st->iters = it_done; st->converged = converged; st->status = status; st->checks = checks;
        st->nF_abs = nF_abs; st->nF_rel = nF_rel; st->nF_ini = nF_ini; st->lambda_min = lmin; st->lambda_max = lmax;
        st->h1 = h1; st->h2 = h2; st->dtau = dtau;
    }
    return status;
}

extern "C" {
int orc_step_v18(double* T, double* P, const double* phc, const double* phv, const double* wN, const double* kmul,
                 double* Vx, double* Vy, double* Vz, orc_v18_params* p, orc_dyrel_stats* st_T, orc_dyrel_stats* st_P,
                 i64 nx, i64 ny, i64 nz) {
    const i64 n = nx * ny * nz, nv = (nx + 1) * (ny + 1) * (nz + 1), nex = (nx + 2) * (ny + 2) * (nz + 2);
    const i64 nfx = (nx + 1) * ny * nz, nfy = nx * (ny + 1) * nz, nfz = nx * ny * (nz + 1);
    const double dx = p->dx, dy = p->dy, dz = p->dz, _dx = 1.0 / dx, _dy = 1.0 / dy, _dz = 1.0 / dz;
    double dt = p->dt;
    const double _dt = 1.0 / dt;
    const double transient = p->it == 0 ? 0.0 : 1.0;
    std::vector<double> Tc0(n), Pc0(n), kv(nv, 1.0), dumc(n, 1.0), kx(nfx), ky(nfy), kz(nfz), rC(n, 0.0), PC(n, 1.0),
        Xc0(n), F(n), F0(n), qx(nfx), qy(nfy), qz(nfz);
    if (p->it == 1)  // introduce the pluton (v18:414-416)
        for (i64 t = 0; t < nex; ++t)
            if (phc[t] == 3.0) T[t] = p->T_pluton;
    orc_InitThermal_dim(Tc0.data(), T, nx, ny, nz);
    orc_InitThermal_dim(Pc0.data(), P, nx, ny, nz);
    int s = ORC_OK;
    if (p->thermal) {  // v18:424-479
        orc_ComputeThermalConductivity(kv.data(), T, phv, p->phi_i, p->sc_kt, p->sc_T, nx, ny, nz);
        orc_SmoothConductivityV2C(dumc.data(), kv.data(), nx, ny, nz);
        orc_SmoothConductivityC2V(kv.data(), dumc.data(), nx, ny, nz);
        orc_InitConductivity(kx.data(), ky.data(), kz.data(), kv.data(), nx, ny, nz);
        orc_ComputeRhoCeffective(rC.data(), T, P, phc, p->phi_i, p->sc_T, p->sc_sigma, p->sc_C, p->sc_rho, nx, ny, nz);
        orc_GershgorinPoisson(Xc0.data(), PC.data(), rC.data(), kx.data(), ky.data(), kz.data(), transient, dt, dx, dy,
                              dz, nx, ny, nz);
        const double lmax = orc_max(Xc0.data(), n);
        s = dyrel_loop(T, F.data(), F0.data(), PC.data(), lmax, &p->thermal_dyrel,
                       [&](double h1, double h2, double dtau) {
                           orc_SetTemperatureBCs_dim(T, ky.data(), wN, phc, p->qyS, _dy, p->Ttop, nx, ny, nz);
                           orc_ComputeFlux(qx.data(), qy.data(), qz.data(), kx.data(), ky.data(), kz.data(), T, _dx,
                                           _dy, _dz, nx, ny, nz);
                           orc_ResidualTemperatureLinearised(F.data(), T, Tc0.data(), rC.data(), phc, PC.data(),
                                                             qx.data(), qy.data(), qz.data(), p->Qt, transient, _dt,
                                                             _dx, _dy, _dz, nx, ny, nz);
                           orc_DYRELUpdate(F0.data(), T, F.data(), h1, h2, dtau, nx, ny, nz);
                       },
                       st_T, nx, ny, nz);
        if (s) return s;
    }
    if (p->hydro) {  // v18:481-538
        orc_ComputeHydroConductivity(kv.data(), T, P, phv, p->ymin, dy, p->k_fact, p->delta, p->sc_sigma, p->sc_T,
                                     p->sc_L, p->sc_t, p->sc_eta, 1, kmul, nx, ny, nz);
        orc_SmoothConductivityV2C(dumc.data(), kv.data(), nx, ny, nz);
        orc_SmoothConductivityC2V(kv.data(), dumc.data(), nx, ny, nz);
        orc_InitConductivity(kx.data(), ky.data(), kz.data(), kv.data(), nx, ny, nz);
        orc_phi_rhof(rC.data(), T, P, phc, p->phi_i, p->sc_rho, p->sc_T, p->sc_sigma, 0, 1, nx, ny, nz);
        orc_GershgorinPoisson(Xc0.data(), PC.data(), rC.data(), kx.data(), ky.data(), kz.data(), transient, dt, dx, dy,
                              dz, nx, ny, nz);
        const double lmax = orc_max(Xc0.data(), n);
        orc_phi_rhof(Xc0.data(), Tc0.data(), Pc0.data(), phc, p->phi_i, p->sc_rho, p->sc_T, p->sc_sigma, 1, 0, nx, ny, nz);
        orc_ComputeFluidDensity(kv.data(), T, P, phv, p->sc_sigma, p->sc_T, p->sc_rho, nx, ny, nz);
        s = dyrel_loop(P, F.data(), F0.data(), PC.data(), lmax, &p->darcy_dyrel,
                       [&](double h1, double h2, double dtau) {
                           orc_phi_rhof(rC.data(), T, P, phc, p->phi_i, p->sc_rho, p->sc_T, p->sc_sigma, 0, 0, nx, ny, nz);
                           orc_SetPressureBCs_dim(P, wN, phc, p->Ptop, nx, ny, nz);
                           orc_ComputeDarcyFlux(qx.data(), qy.data(), qz.data(), kv.data(), kx.data(), ky.data(),
                                                kz.data(), P, p->g, _dx, _dy, _dz, nx, ny, nz);
                           orc_ResidualFluidPressure(F.data(), phc, rC.data(), Xc0.data(), PC.data(), qx.data(),
                                                     qy.data(), qz.data(), transient, _dt, _dx, _dy, _dz, nx, ny, nz);
                           orc_DYRELUpdate(F0.data(), P, F.data(), h1, h2, dtau, nx, ny, nz);
                       },
                       st_P, nx, ny, nz);
        if (s) return s;
    }
    // velocity (v18:543-548): k/mu, smoothed, and the Darcy flux
    orc_ComputeHydroConductivity(kv.data(), T, P, phv, p->ymin, dy, p->k_fact, p->delta, p->sc_sigma, p->sc_T, p->sc_L,
                                 p->sc_t, p->sc_eta, 2, kmul, nx, ny, nz);
    orc_SmoothConductivityV2C(dumc.data(), kv.data(), nx, ny, nz);
    orc_SmoothConductivityC2V(kv.data(), dumc.data(), nx, ny, nz);
    orc_InitConductivity(kx.data(), ky.data(), kz.data(), kv.data(), nx, ny, nz);
    orc_ComputeFluidDensity(kv.data(), T, P, phv, p->sc_sigma, p->sc_T, p->sc_rho, nx, ny, nz);
    orc_ComputeDarcyFlux(Vx, Vy, Vz, kv.data(), kx.data(), ky.data(), kz.data(), P, p->g, _dx, _dy, _dz, nx, ny, nz);
    p->n_adv = 0;
    if (p->it > 0) {  // v18:550-572
        p->time += dt;
        if (p->advection) {
            const double vmax = std::max(std::max(orc_max_abs(Vx, nfx), orc_max_abs(Vy, nfy)), orc_max_abs(Vz, nfz));
            const double dt_adv = p->C_adv * 1.0 / 6.1 * std::min(std::min(dx, dy), dz) / vmax;
            const int bt[6] = {0, 0, 1, 1, 0, 0};
            const double bv[6] = {0.0, 0.0, p->Tbot, p->Ttop, 0.0, 0.0};
            const int quirk = p->weno_variant == 1;
            if (!p->dt_constant) {
                p->dt = dt_adv;
                orc_AdvectWithWeno5_v2(T, Vx, Vy, Vz, p->dt, _dx, _dy, _dz, bt, bv, quirk, nx, ny, nz);
                p->n_adv = 1;
            } else {
                const double na = std::ceil(dt / dt_adv);
                if (!(na >= 1.0 && na <= 32767.0)) return 1;  // Int16(ceil(dt/dt_adv)) would throw
                const int nt_adv = (int)na;
                const double dt_adv1 = dt / nt_adv;
                for (int ia = 0; ia < nt_adv; ++ia)
                    orc_AdvectWithWeno5_v2(T, Vx, Vy, Vz, dt_adv1, _dx, _dy, _dz, bt, bv, quirk, nx, ny, nz);
                p->n_adv = nt_adv;
            }
        }
    }
    return ORC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// SetInitialConditions_Khaled (Dimensional/HydroThermal3D_v18.jl:59-129) and
// Topography (v18.jl:43-57): phases, T and P of the dimensional model's
// detachment-fault geometry.  The grid coordinates are the driver's
// (v18.jl:355-367): ghosted cell centres xce = LinRange(xmin-dx/2, xmax+dx/2,
// nx+2), vertices xv = LinRange(xmin, xmax, nx+1); Julia evaluates element i
// of LinRange(a, b, n) as (1-t)*a + t*b with t = i/(n-1).
// ---------------------------------------------------------------------------
extern "C" {

struct orc_khaled_geom {      // the driver's `geometry` NamedTuple (v18.jl:236-287)
    double y_plateau;
    double surf_a1, surf_b1;
    double fault[4][6];       // detachment, fault1, fault2, fault3: a1, b1, a2, b2, a3, b3
};

static double orc_linrange(double a, double b, i64 n, i64 i) {
    const double t = (double)i / (double)(n - 1);
    return (1.0 - t) * a + t * b;
}

static double orc_topography(double x, double y_plateau, double a2, double b2) {
    const double xW = -b2 / a2;
    const double xE = (y_plateau - b2) / a2;
    if (x <= xW) return 0.0;
    if (x >= xE) return y_plateau;
    return a2 * x + b2;
}

static double orc_khaled_phase(double x, double y, double z, double y0, const orc_khaled_geom* g, double L,
                               double zmax) {
    double ph = 0.0;  // crust
    for (int f = 0; f < 4; ++f) {
        const double* c = g->fault[f];
        if (y < (x * c[0] + c[1]) && y > (x * c[2] + c[3]) && y > (x * c[4] + c[5])) ph = 2.0;
    }
    // pluton: an ellipsoid rotated by 60 degrees in the x-y plane
    const double a = 1e3 / L, b = 10e3 / L, cz = 500e3 / L, z0 = zmax / 2;
    const double x0 = 53057.07323 / L, yp = -8992.45195 / L;
    const double t_ta = 60 * (M_PI / 180);
    const double u = ((x - x0) * cos(t_ta) - (y - yp) * sin(t_ta)) / a;
    const double v = ((x - x0) * sin(t_ta) + (y - yp) * cos(t_ta)) / b;
    const double w = (z - z0) / cz;
    if (u * u + v * v + w * w < 1) ph = 3.0;
    const double tiny = 1e-9;
    if (y > (y0 - tiny)) ph = 1.0;  // air
    return ph;
}

void orc_SetInitialConditions_Khaled(double* phc, double* phv, double* wN, const orc_khaled_geom* g, double* Tc_ex,
                                     double* Pc_ex, double Tbot, double Ttop, double Pbot, double Ptop, double xmin,
                                     double ymin, double zmin, double xmax, double ymax, double zmax, double L, i64 nx,
                                     i64 ny, i64 nz) {
    (void)wN;  // the weight loop looks for phase -1, which is never assigned: wN keeps its values
    const double dx = (xmax - xmin) / nx, dy = (ymax - ymin) / ny, dz = (zmax - zmin) / nz;
    const i64 n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    auto xce = [&](i64 i) { return orc_linrange(xmin - dx / 2, xmax + dx / 2, n1, i); };
    auto yce = [&](i64 j) { return orc_linrange(ymin - dy / 2, ymax + dy / 2, n2, j); };
    auto zce = [&](i64 k) { return orc_linrange(zmin - dz / 2, zmax + dz / 2, n3, k); };
    // vertices
    for (i64 k = 0; k <= nz; ++k)
        for (i64 j = 0; j <= ny; ++j)
            for (i64 i = 0; i <= nx; ++i) {
                const double x = orc_linrange(xmin, xmax, nx + 1, i), y = orc_linrange(ymin, ymax, ny + 1, j),
                             z = orc_linrange(zmin, zmax, nz + 1, k);
                const double y0 = orc_topography(x, g->y_plateau, g->surf_a1, g->surf_b1);
                phv[i + (nx + 1) * (j + (ny + 1) * k)] = orc_khaled_phase(x, y, z, y0, g, L, zmax);
            }
    // cells (ghosted): phases, then T and P as the sequence of whole-array statements
    const double y_bot = -30e3 / L;
    auto profile = [&](double V0top, double Vbot, i64 i, i64 j) {
        const double y0 = orc_topography(xce(i), g->y_plateau, g->surf_a1, g->surf_b1);
        const double dVdy = (V0top - Vbot) / (y0 - y_bot);
        return V0top + dVdy * (yce(j) - y0);
    };
    auto field = [&](double Vtop, double Vbot, i64 i, i64 j, i64 k) {
        // V = profile; x ghosts copy; y ghosts Dirichlet (2 Vbot / 2 Vtop - inner); z: last plane copies
        auto vx = [&](i64 ii, i64 jj) { return profile(Vtop, Vbot, ii == 0 ? 1 : (ii == n1 - 1 ? n1 - 2 : ii), jj); };
        auto vy = [&](i64 ii, i64 jj) {
            if (jj == 0) return 2 * Vbot - vx(ii, 1);
            if (jj == n2 - 1) return 2 * Vtop - vx(ii, n2 - 2);
            return vx(ii, jj);
        };
        (void)k;  // the profile does not depend on z; the z-ghost statements copy equal values
        double v = vy(i, j);
        const double x = xce(i), y = yce(j);
        if ((y > 0 && (y > (x * g->surf_a1 + g->surf_b1))) || y > g->y_plateau) v = Vtop;
        return v;
    };
    for (i64 k = 0; k < n3; ++k)
        for (i64 j = 0; j < n2; ++j)
            for (i64 i = 0; i < n1; ++i) {
                const i64 e = i + n1 * (j + n2 * k);
                const double x = xce(i), y = yce(j), z = zce(k);
                const double y0 = orc_topography(x, g->y_plateau, g->surf_a1, g->surf_b1);
                phc[e] = orc_khaled_phase(x, y, z, y0, g, L, zmax);
                Tc_ex[e] = field(Ttop, Tbot, i, j, k);
                Pc_ex[e] = field(Ptop, Pbot, i, j, k);
            }
}

}  // extern "C"

// ===========================================================================
// Output diagnostics, Dimensional/kernels_HT3D_postprocessing.jl, and the
// Nusselt number of Dimensionless/HydroThermal3D_Alban_v6.jl:345-348.
// Every output is a cell array (nx,ny,nz); cells whose phase phc_ex is 1
// (air) get NaN, except where the reference leaves them untouched (the Y/Z
// components of Velocity!, and EffectiveHeatCapacity!).
// ===========================================================================
extern "C" {

#define POST_LOOP                                                                         \
    A3 phc = mk((double*)phc_ex_, nx + 2, ny + 2, nz + 2);                                \
    PARFOR3(nx, ny, nz)
#define POST_AIR (phc(i + 1, j + 1, k + 1) == 1.0)
#define POST_PH phc(i + 1, j + 1, k + 1)
#define POST_OUT(X_) X_[i + nx * (j + ny * k)]

// Phase!  :1-10
void orc_Phase(double* X, const double* phc_ex_, i64 nx, i64 ny, i64 nz) {
    POST_LOOP { POST_OUT(X) = POST_AIR ? NAN : POST_PH; }
}
// Pressure!  :12-21
void orc_Pressure(double* X, const double* Pc_ex_, const double* phc_ex_, double scale_s, i64 nx, i64 ny, i64 nz) {
    A3 Pc = mk((double*)Pc_ex_, nx + 2, ny + 2, nz + 2);
    POST_LOOP { POST_OUT(X) = POST_AIR ? NAN : Pc(i + 1, j + 1, k + 1) * scale_s; }
}
// Temperature!  :23-32
void orc_Temperature(double* X, const double* Tc_ex_, const double* phc_ex_, double scale_T, i64 nx, i64 ny, i64 nz) {
    A3 Tc = mk((double*)Tc_ex_, nx + 2, ny + 2, nz + 2);
    POST_LOOP { POST_OUT(X) = POST_AIR ? NAN : Tc(i + 1, j + 1, k + 1) * scale_T; }
}
// Velocity!  :34-45 -- face averages to centres; air sets only X
void orc_Velocity(double* X, double* Y, double* Z, const double* Vx_, const double* Vy_, const double* Vz_,
                  const double* phc_ex_, double scale_V, i64 nx, i64 ny, i64 nz) {
    A3 Vx = mk((double*)Vx_, nx + 1, ny, nz), Vy = mk((double*)Vy_, nx, ny + 1, nz), Vz = mk((double*)Vz_, nx, ny, nz + 1);
    POST_LOOP {
        if (!POST_AIR) {
            POST_OUT(X) = 0.5 * (Vx(i, j, k) + Vx(i + 1, j, k)) * scale_V;
            POST_OUT(Y) = 0.5 * (Vy(i, j, k) + Vy(i, j + 1, k)) * scale_V;
            POST_OUT(Z) = 0.5 * (Vz(i, j, k) + Vz(i, j, k + 1)) * scale_V;
        } else {
            POST_OUT(X) = NAN;
        }
    }
}
// EffectiveThermalConductivity!  :47-57
void orc_EffectiveThermalConductivity(double* X, const double* Tc_ex_, double phi0, const double* phc_ex_,
                                      double scale_T, i64 nx, i64 ny, i64 nz) {
    A3 Tc = mk((double*)Tc_ex_, nx + 2, ny + 2, nz + 2);
    POST_LOOP {
        if (!POST_AIR) {
            const double T = Tc(i + 1, j + 1, k + 1) * scale_T;
            POST_OUT(X) = ((1.0 - phi_of(POST_PH, phi0)) * kTs(T) + phi_of(POST_PH, phi0) * kTf(T));
        } else {
            POST_OUT(X) = NAN;
        }
    }
}
// EffectiveHeatCapacity!  :60-70 -- solid heat capacity only; air untouched
// (Pc_ex, phi_i and the sigma/C/rho scales are accepted and unused, as there)
void orc_EffectiveHeatCapacity(double* X, const double* Tc_ex_, const double* Pc_ex_, const double* phc_ex_,
                               double phi_i, double sca_T, double sca_s, double sca_C, double sca_rho, i64 nx, i64 ny,
                               i64 nz) {
    (void)Pc_ex_, (void)phi_i, (void)sca_s, (void)sca_C, (void)sca_rho;
    A3 Tc = mk((double*)Tc_ex_, nx + 2, ny + 2, nz + 2);
    POST_LOOP {
        if (!POST_AIR) POST_OUT(X) = Cs(Tc(i + 1, j + 1, k + 1) * sca_T);
    }
}
// Permeability!  :72-85 -- y of the cell centre; fault phase (2) scaled by k_fact
void orc_Permeability(double* X, double k_fact, double ymin, double dy, const double* phc_ex_, double delta,
                      double scale_L, i64 nx, i64 ny, i64 nz) {
    POST_LOOP {
        if (!POST_AIR) {
            const double y = ymin + (double)j * dy + dy / 2;
            double v = k_F(y * scale_L, delta * scale_L);
            if (POST_PH == 2.0) v *= k_fact;
            POST_OUT(X) = v;
        } else {
            POST_OUT(X) = NAN;
        }
    }
}
// FluidDensity!  :87-98
void orc_FluidDensity(double* X, const double* Tc_ex_, const double* Pc_ex_, const double* phc_ex_, double scale_T,
                      double scale_s, i64 nx, i64 ny, i64 nz) {
    A3 Tc = mk((double*)Tc_ex_, nx + 2, ny + 2, nz + 2), Pc = mk((double*)Pc_ex_, nx + 2, ny + 2, nz + 2);
    POST_LOOP {
        if (!POST_AIR) {
            const double T = Tc(i + 1, j + 1, k + 1) * scale_T - 273.15;
            const double P = Pc(i + 1, j + 1, k + 1) * scale_s;
            POST_OUT(X) = rhof_C(T, P);
        } else {
            POST_OUT(X) = NAN;
        }
    }
}
// Viscosity!  :100-109
void orc_Viscosity(double* X, const double* Tc_ex_, const double* phc_ex_, double scale_T, i64 nx, i64 ny, i64 nz) {
    A3 Tc = mk((double*)Tc_ex_, nx + 2, ny + 2, nz + 2);
    POST_LOOP { POST_OUT(X) = POST_AIR ? NAN : mu_f(Tc(i + 1, j + 1, k + 1) * scale_T); }
}
// Peclet!  :111-129 -- L rho_f C_f |V| / k_eff; x^2 is x*x (Julia literal power)
void orc_Peclet(double* X, const double* Tc_ex_, const double* Pc_ex_, const double* Vx_, const double* Vy_,
                const double* Vz_, const double* phc_ex_, double phi0, double scale_T, double scale_s, double scale_V,
                double scale_L, i64 nx, i64 ny, i64 nz) {
    A3 Tc = mk((double*)Tc_ex_, nx + 2, ny + 2, nz + 2), Pc = mk((double*)Pc_ex_, nx + 2, ny + 2, nz + 2);
    A3 Vx = mk((double*)Vx_, nx + 1, ny, nz), Vy = mk((double*)Vy_, nx, ny + 1, nz), Vz = mk((double*)Vz_, nx, ny, nz + 1);
    POST_LOOP {
        if (!POST_AIR) {
            const double x = 0.5 * (Vx(i, j, k) + Vx(i + 1, j, k)) * scale_V;
            const double y = 0.5 * (Vy(i, j, k) + Vy(i, j + 1, k)) * scale_V;
            const double z = 0.5 * (Vz(i, j, k) + Vz(i, j, k + 1)) * scale_V;
            const double V = std::sqrt(x * x + y * y + z * z);
            const double T = Tc(i + 1, j + 1, k + 1) * scale_T;
            const double P = Pc(i + 1, j + 1, k + 1) * scale_s;
            const double rho = rhof_C(T - 273.15, P);
            const double C = Cf(T);
            const double keff = ((1 - phi_of(POST_PH, phi0)) * kTs(T) + phi_of(POST_PH, phi0) * kTf(T));
            POST_OUT(X) = scale_L * rho * C * V / keff;
        } else {
            POST_OUT(X) = NAN;
        }
    }
}
#undef POST_LOOP
#undef POST_AIR
#undef POST_PH
#undef POST_OUT

// Nu = sum(qy[:,end,:]) / (Lx*Lz) / (nx*nz), Dimensionless/HydroThermal3D_Alban_v6.jl:345-348.
// qy is (nx, ny+1, nz); the top-face values are summed in the canonical tree
// order over the (i fastest, then k) linear index of the face.
double orc_Nusselt(const double* qy, double Lx, double Lz, i64 nx, i64 ny, i64 nz) {
    std::vector<double> face((size_t)(nx * nz));
    for (i64 k = 0; k < nz; ++k)
        for (i64 i = 0; i < nx; ++i) face[(size_t)(i + nx * k)] = qy[i + nx * (ny + (ny + 1) * k)];
    return tree_sum(face.data(), nx * nz) / (Lx * Lz) / (double)(nx * nz);
}

}  // extern "C"
