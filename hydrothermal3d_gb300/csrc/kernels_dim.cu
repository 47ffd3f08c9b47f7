// Per-kernel drop-ins for the dimensional reference kernels
// (Dimensional/kernels_HT3D_dimensional.jl) and the material laws of
// Dimensional/HydroThermal3D_v18.jl:29-39.  Compiled with -fmad=false; each
// expression keeps the reference's evaluation order.
#include "ht3d_internal.cuh"
#include "laws.cuh"

#define GIDX                                             \
    const int i = blockIdx.x * blockDim.x + threadIdx.x; \
    const int j = blockIdx.y * blockDim.y + threadIdx.y; \
    const int k = blockIdx.z * blockDim.z + threadIdx.z

#define EXI(i, j, k) ix3(i, j, k, nx + 2, ny + 2)
#define VXI(i, j, k) ix3(i, j, k, nx + 1, ny + 1)
#define CI(i, j, k) ix3(i, j, k, nx, ny)

namespace {

// 8-point average of an extended centre field at vertex (i,j,k)
// (Dimensional/kernels_HT3D_dimensional.jl:43-45)
__device__ __forceinline__ double vtx8(const double* __restrict__ A, int i, int j, int k, int nx, int ny) {
    double v = 1.0 / 8.0 * (A[EXI(i + 1, j + 1, k + 1)] + A[EXI(i + 1, j, k + 1)] + A[EXI(i, j + 1, k + 1)] + A[EXI(i, j, k + 1)]);
    v += 1.0 / 8.0 * (A[EXI(i + 1, j + 1, k + 0)] + A[EXI(i + 1, j, k + 0)] + A[EXI(i, j + 1, k + 0)] + A[EXI(i, j, k + 0)]);
    return v;
}

__global__ void k_thermal_conductivity(double* ktv, const double* __restrict__ Tce, const double* __restrict__ phv,
                                       double phi0, double scale_kt, double scale_T, int nx, int ny, int nz) {
    GIDX;
    if (i > nx || j > ny || k > nz) return;
    double Tv = vtx8(Tce, i, j, k, nx, ny);
    Tv *= scale_T;
    const double ph = phv[VXI(i, j, k)];
    ktv[VXI(i, j, k)] = ((1 - law_phi(ph, phi0)) * law_kTs(Tv) + law_phi(ph, phi0) * law_kTf(Tv)) / scale_kt;
}

__global__ void k_hydro_conductivity(double* kfv, const double* __restrict__ Tce, const double* __restrict__ Pce,
                                     const double* __restrict__ phv, double ymin, double dy, double k_fact, double delta,
                                     double sc_s, double sc_T, double sc_L, double sc_t, double sc_eta, int mode,
                                     const double* __restrict__ kmul, int nx, int ny, int nz) {
    GIDX;
    if (i > nx || j > ny || k > nz) return;
    double Tv = vtx8(Tce, i, j, k, nx, ny);
    Tv *= sc_T;
    if (Tv < 293.15) Tv = 293.15;
    double Pv = vtx8(Pce, i, j, k, nx, ny);
    Pv *= sc_s;
    const double y = ymin + (double)j * dy;
    double kF = law_kF(y * sc_L, delta * sc_L);
    if (kmul) kF *= kmul[VXI(i, j, k)];
    const int v = VXI(i, j, k);
    const double rk_mu = law_rhof_C(Tv - 273.15, Pv) * kF / law_muf(Tv);
    double out = kfv[v];
    if (mode == 1) out = rk_mu / sc_t;
    else if (mode == 2) out = (kF / law_muf(Tv)) / (sc_L * sc_L / sc_eta);
    else if (mode == 3) out = kF / (sc_L * sc_L);
    if (ph_eq(phv[v], 2.0)) out *= k_fact;
    kfv[v] = out;
}

__global__ void k_fluid_density(double* rfv, const double* __restrict__ Tce, const double* __restrict__ Pce,
                                const double* __restrict__ phv, double sc_s, double sc_T, double sc_rho, int nx, int ny,
                                int nz) {
    GIDX;
    if (i > nx || j > ny || k > nz) return;
    double Tv = vtx8(Tce, i, j, k, nx, ny);
    Tv *= sc_T;
    double Pv = vtx8(Pce, i, j, k, nx, ny);
    Pv *= sc_s;
    const int v = VXI(i, j, k);
    double r = law_rhof_C(Tv - 273.15, Pv) / sc_rho;
    if (ph_eq(phv[v], 1.0)) r = 0.000 / sc_rho;
    rfv[v] = r;
}

// SmoothConductivityV2C  :111-114  ktc <- av(ktv)
__global__ void k_smooth_v2c(double* ktc, const double* __restrict__ kv, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    ktc[CI(i, j, k)] = (kv[VXI(i, j, k)] + kv[VXI(i + 1, j, k)] + kv[VXI(i, j + 1, k)] + kv[VXI(i + 1, j + 1, k)] +
                        kv[VXI(i, j, k + 1)] + kv[VXI(i + 1, j, k + 1)] + kv[VXI(i, j + 1, k + 1)] +
                        kv[VXI(i + 1, j + 1, k + 1)]) * 0.125;
}
// SmoothConductivityC2V  :116-119  inn(ktv) <- av(ktc)
__global__ void k_smooth_c2v(double* kv, const double* __restrict__ c, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx - 1 || j >= ny - 1 || k >= nz - 1) return;
    kv[VXI(i + 1, j + 1, k + 1)] = (c[CI(i, j, k)] + c[CI(i + 1, j, k)] + c[CI(i, j + 1, k)] + c[CI(i + 1, j + 1, k)] +
                                    c[CI(i, j, k + 1)] + c[CI(i + 1, j, k + 1)] + c[CI(i, j + 1, k + 1)] +
                                    c[CI(i + 1, j + 1, k + 1)]) * 0.125;
}
// InitConductivity!  :133-138
__global__ void k_init_conductivity(double* kx, double* ky, double* kz, const double* __restrict__ kv, int nx, int ny,
                                    int nz) {
    GIDX;
    if (i < nx + 1 && j < ny && k < nz)
        kx[ix3(i, j, k, nx + 1, ny)] = (kv[VXI(i, j, k)] + kv[VXI(i, j + 1, k)] + kv[VXI(i, j, k + 1)] + kv[VXI(i, j + 1, k + 1)]) * 0.25;
    if (i < nx && j < ny + 1 && k < nz)
        ky[ix3(i, j, k, nx, ny + 1)] = (kv[VXI(i, j, k)] + kv[VXI(i + 1, j, k)] + kv[VXI(i, j, k + 1)] + kv[VXI(i + 1, j, k + 1)]) * 0.25;
    if (i < nx && j < ny && k < nz + 1)
        kz[ix3(i, j, k, nx, ny)] = (kv[VXI(i, j, k)] + kv[VXI(i + 1, j, k)] + kv[VXI(i, j + 1, k)] + kv[VXI(i + 1, j + 1, k)]) * 0.25;
}
// ComputeρCeffective!  :148-160
__global__ void k_rhoC_eff(double* rC, const double* __restrict__ T, const double* __restrict__ P,
                           const double* __restrict__ phc, double phii, double sT, double ss, double sC, double srho,
                           int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const int e = EXI(i + 1, j + 1, k + 1);
    const double ph = phc[e];
    if (!ph_abs_eq(ph, 1.0)) {
        const double Tsca = T[e] * sT, Psca = P[e] * ss;
        const double r_eff = law_phi(ph, phii) * law_rhof_C(Tsca - 273.15, Psca) + (1.0 - law_phi(ph, phii)) * law_rhos(Tsca);
        const double Ceff = law_phi(ph, phii) * law_Cf(Tsca) + (1.0 - law_phi(ph, phii)) * law_Cs(Tsca);
        rC[CI(i, j, k)] = (r_eff * Ceff) / srho / sC;
    }
}
// ResidualTemperatureLinearised!  :162-181
__global__ void k_res_temperature(double* F, const double* __restrict__ T, const double* __restrict__ T0,
                                  const double* __restrict__ rC, const double* __restrict__ phc,
                                  const double* __restrict__ PC, const double* __restrict__ qx,
                                  const double* __restrict__ qy, const double* __restrict__ qz, double Qt,
                                  double transient, double _dt, double _dx, double _dy, double _dz, int nx, int ny,
                                  int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const int e = EXI(i + 1, j + 1, k + 1), c = CI(i, j, k);
    const double ph = phc[e];
    if (!ph_abs_eq(ph, 1.0)) {
        double Q = 0.;
        if (ph_eq(ph, 3.0)) Q = Qt;
        double f = transient * rC[c] * _dt * (T[e] - T0[c]);
        f += (qx[ix3(i + 1, j, k, nx + 1, ny)] - qx[ix3(i, j, k, nx + 1, ny)]) * _dx;
        f += (qy[ix3(i, j + 1, k, nx, ny + 1)] - qy[ix3(i, j, k, nx, ny + 1)]) * _dy;
        f += (qz[ix3(i, j, k + 1, nx, ny)] - qz[ix3(i, j, k, nx, ny)]) * _dz;
        f -= transient * Q;
        f /= PC[c];
        F[c] = f;
    } else {
        F[c] = 0.;
    }
}
// SetTemperatureBCs! (:183-205) / SetPressureBCs! (:291-314) in place, with
// snapshot semantics (every rule reads cells as they were before the call;
// a later rule of one cell overrides an earlier one) in two passes over the
// phase array: MODE bit 1 clear evaluates the new value of each written cell
// from X, which this pass does not modify, into B; MODE bit 1 set stores B
// into X for the same cells.  MODE bit 0: pressure (1) or temperature (0).
template <int MODE>
__global__ void k_dim_bcs(double* X, double* B, const double* __restrict__ ky, const double* __restrict__ wN,
                          const double* __restrict__ ph, double qyS, double _dy, double VN, int nx, int ny, int nz) {
    constexpr int PRESSURE = MODE & 1, APPLY = MODE >> 1;
    const int n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    const int k0 = blockIdx.z * kZPer;  // grid3z launch: kZPer planes of one (i, j) column
    double pv[kZPer];                   // the column's phase codes, loaded before any rule runs
#pragma unroll
    for (int kk = 0; kk < kZPer; ++kk) pv[kk] = k0 + kk < n3 ? ph[EXI(i, j, k0 + kk)] : 0.0;
#pragma unroll
    for (int kk = 0; kk < kZPer; ++kk) {
        const int k = k0 + kk;
        if (k >= n3) break;
        const int e = EXI(i, j, k);
        const double p = pv[kk];
        const int kmaxx = PRESSURE ? n3 - 2 : n3 - 1;  // x-rule z range differs between the two kernels
        const bool xl = i == 0 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= kmaxx;
        const bool xr = i == n1 - 1 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= kmaxx;
        const bool ys = j == 0 && i >= 1 && i <= n1 - 2 && k >= 1 && k <= n3 - 2;
        const bool imm = ph_eq(p, -1.0) && j >= 1;
        const bool zb = k == 0 && i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2;
        const bool zf = k == n3 - 1 && i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2;
        const bool air = ph_eq(p, 1.0);
        if (!(air || xl || xr || ys || imm || zb || zf)) continue;
        if (APPLY) {
            X[e] = B[e];
            continue;
        }
        double v = 0.0;
        if (air) v = VN;
        if (xl) v = X[EXI(1, j, k)];
        if (xr) v = X[EXI(n1 - 2, j, k)];
        if (ys) {
            if (PRESSURE) v = X[EXI(i, 1, k)];
            else v = qyS / _dy / ky[ix3(i - 1, 0, k - 1, nx, ny + 1)] + X[EXI(i, 1, k)];
        }
        if (imm) {
            const double wn = wN[i + (nx + 2) * k];
            v = (VN - (1.0 - wn) * X[EXI(i, j - 1, k)]) / wn;
        }
        if (zb) v = X[EXI(i, j, 1)];
        if (zf) v = X[EXI(i, j, n3 - 2)];
        B[e] = v;
    }
}
// ϕρf (:225-235), ϕρf_old (:237-247, cell inputs), ϕdρdP! (:249-259)
__global__ void k_phi_rhof(double* out, const double* __restrict__ T, const double* __restrict__ P,
                           const double* __restrict__ phc, double phii, double srho, double sT, double ss, int cell_in,
                           int deriv, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const double ph = phc[EXI(i + 1, j + 1, k + 1)];
    if (!ph_eq(ph, 1.0)) {
        const int s = cell_in ? CI(i, j, k) : EXI(i + 1, j + 1, k + 1);
        const double Tc = T[s] * sT - 273.15;
        const double Pc = P[s] * ss;
        out[CI(i, j, k)] = deriv ? law_phi(ph, phii) * law_drhodP_C(Tc, Pc) / (srho / ss)
                                 : law_phi(ph, phii) * law_rhof_C(Tc, Pc) / srho;
    }
}
// ComputeDarcyFlux!  :266-272
__global__ void k_darcy_flux(double* qx, double* qy, double* qz, const double* __restrict__ rfv,
                             const double* __restrict__ kx, const double* __restrict__ ky,
                             const double* __restrict__ kz, const double* __restrict__ P, double g, double _dx,
                             double _dy, double _dz, int nx, int ny, int nz) {
    GIDX;
    if (i < nx + 1 && j < ny && k < nz) {
        const int f = ix3(i, j, k, nx + 1, ny);
        qx[f] = -kx[f] * (_dx * (P[EXI(i + 1, j + 1, k + 1)] - P[EXI(i, j + 1, k + 1)]));
    }
    if (i < nx && j < ny + 1 && k < nz) {
        const int f = ix3(i, j, k, nx, ny + 1);
        const double av = (rfv[VXI(i, j, k)] + rfv[VXI(i + 1, j, k)] + rfv[VXI(i, j, k + 1)] + rfv[VXI(i + 1, j, k + 1)]) * 0.25;
        qy[f] = -ky[f] * (_dy * (P[EXI(i + 1, j + 1, k + 1)] - P[EXI(i + 1, j, k + 1)]) - g * av);
    }
    if (i < nx && j < ny && k < nz + 1) {
        const int f = ix3(i, j, k, nx, ny);
        qz[f] = -kz[f] * (_dz * (P[EXI(i + 1, j + 1, k + 1)] - P[EXI(i + 1, j + 1, k)]));
    }
}
// ResidualFluidPressure!  :274-289
__global__ void k_res_pressure(double* F, const double* __restrict__ phc, const double* __restrict__ prf,
                               const double* __restrict__ prf0, const double* __restrict__ PC,
                               const double* __restrict__ qx, const double* __restrict__ qy,
                               const double* __restrict__ qz, double transient, double _dt, double _dx, double _dy,
                               double _dz, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const int c = CI(i, j, k);
    const double ph = phc[EXI(i + 1, j + 1, k + 1)];
    if (!ph_abs_eq(ph, 1.0)) {
        double f = transient * _dt * (prf[c] - prf0[c]);
        f += (qx[ix3(i + 1, j, k, nx + 1, ny)] - qx[ix3(i, j, k, nx + 1, ny)]) * _dx;
        f += (qy[ix3(i, j + 1, k, nx, ny + 1)] - qy[ix3(i, j, k, nx, ny + 1)]) * _dy;
        f += (qz[ix3(i, j, k + 1, nx, ny)] - qz[ix3(i, j, k, nx, ny)]) * _dz;
        f /= PC[c];
        F[c] = f;
    } else {
        F[c] = 0.;
    }
}
// Init_vel! (dimensional)  :328-333
__global__ void k_init_vel_dim(double* Vx, double* Vy, double* Vz, const double* __restrict__ qx,
                               const double* __restrict__ qy, const double* __restrict__ qz,
                               const double* __restrict__ rfv, int nx, int ny, int nz) {
    GIDX;
    if (i < nx + 1 && j < ny && k < nz) {
        const int f = ix3(i, j, k, nx + 1, ny);
        Vx[f] = qx[f] / ((rfv[VXI(i, j, k)] + rfv[VXI(i, j + 1, k)] + rfv[VXI(i, j, k + 1)] + rfv[VXI(i, j + 1, k + 1)]) * 0.25);
    }
    if (i < nx && j < ny + 1 && k < nz) {
        const int f = ix3(i, j, k, nx, ny + 1);
        Vy[f] = qy[f] / ((rfv[VXI(i, j, k)] + rfv[VXI(i + 1, j, k)] + rfv[VXI(i, j, k + 1)] + rfv[VXI(i + 1, j, k + 1)]) * 0.25);
    }
    if (i < nx && j < ny && k < nz + 1) {
        const int f = ix3(i, j, k, nx, ny);
        Vz[f] = qz[f] / ((rfv[VXI(i, j, k)] + rfv[VXI(i + 1, j, k)] + rfv[VXI(i, j + 1, k)] + rfv[VXI(i + 1, j + 1, k)]) * 0.25);
    }
}
__global__ void k_law_eval(double* out, const double* __restrict__ a, const double* __restrict__ b, int which, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = law_eval(which, a[t], b ? b[t] : 0.0);
}

}  // namespace

extern "C" {

#define G3(a, b, c) grid3((a), (b), (c), kBlock3)
#define DIMS ht3d_check_dims(nx, ny, nz, 1)

int ht3d_ComputeThermalConductivity(ht3d_ctx* ctx, double* ktv, const double* Tce, const double* phv, double phi0,
                                    double scale_kt, double scale_T, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(ktv, Tce, phv), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_thermal_conductivity, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, ktv, Tce, phv, phi0, scale_kt,
                    scale_T, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ComputeHydroConductivity(ht3d_ctx* ctx, double* kfv, const double* Tce, const double* Pce, const double* phv,
                                  double ymin, double dy, double k_fact, double delta, double scale_sigma,
                                  double scale_T, double scale_L, double scale_t, double scale_eta, int mode,
                                  const double* kmul_v, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(kfv, Tce, Pce, phv), "null argument");
        DIMS;
        HT3D_REQUIRE(mode >= 1 && mode <= 3, "mode must be 1, 2 or 3");
        HT3D_LAUNCH(ctx, k_hydro_conductivity, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, kfv, Tce, Pce, phv, ymin, dy,
                    k_fact, delta, scale_sigma, scale_T, scale_L, scale_t, scale_eta, mode, kmul_v, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ComputeFluidDensity(ht3d_ctx* ctx, double* rhofv, const double* Tce, const double* Pce, const double* phv,
                             double scale_sigma, double scale_T, double scale_rho, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(rhofv, Tce, Pce, phv), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_fluid_density, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, rhofv, Tce, Pce, phv, scale_sigma,
                    scale_T, scale_rho, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_SmoothConductivityV2C(ht3d_ctx* ctx, double* ktc, const double* ktv, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(ktc, ktv), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_smooth_v2c, G3(nx, ny, nz), kBlock3, 0, ktc, ktv, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_SmoothConductivityC2V(ht3d_ctx* ctx, double* ktv, const double* ktc, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(ktv, ktc), "null argument");
        DIMS;
        if (nx > 1 && ny > 1 && nz > 1)
            HT3D_LAUNCH(ctx, k_smooth_c2v, G3(nx - 1, ny - 1, nz - 1), kBlock3, 0, ktv, ktc, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_InitConductivity(ht3d_ctx* ctx, double* kx, double* ky, double* kz, const double* ktv, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(kx, ky, kz, ktv), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_init_conductivity, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, kx, ky, kz, ktv, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ComputeRhoCeffective(ht3d_ctx* ctx, double* rhoC_eff, const double* Tc_ex, const double* Pc_ex,
                              const double* phc_ex, double phi_i, double sca_T, double sca_sigma, double sca_C,
                              double sca_rho, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(rhoC_eff, Tc_ex, Pc_ex, phc_ex), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_rhoC_eff, G3(nx, ny, nz), kBlock3, 0, rhoC_eff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma,
                    sca_C, sca_rho, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ResidualTemperatureLinearised(ht3d_ctx* ctx, double* F, const double* Tc_ex, const double* Tc_old,
                                       const double* rhoC_eff, const double* phc_ex, const double* PC,
                                       const double* qx, const double* qy, const double* qz, double Qt,
                                       double transient, double _dt, double _dx, double _dy, double _dz, int nx,
                                       int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(F, Tc_ex, Tc_old, rhoC_eff, phc_ex, PC, qx, qy, qz), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_res_temperature, G3(nx, ny, nz), kBlock3, 0, F, Tc_ex, Tc_old, rhoC_eff, phc_ex, PC, qx, qy,
                    qz, Qt, transient, _dt, _dx, _dy, _dz, nx, ny, nz);
        return HT3D_OK;
    });
}

static int dim_bcs(ht3d_ctx* ctx, int pressure, double* X, const double* ky, const double* wN, const double* phc,
                   double qyS, double _dy, double VN, int nx, int ny, int nz) {
    DIMS;
    HT3D_REQUIRE(X && wN && phc && (pressure || ky), "null argument");
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    double* B = (double*)ht3d_scratch(ctx, SLOT_SNAP, sizeof(double) * nex);
    const dim3 g = grid3z(nx + 2, ny + 2, nz + 2);
    if (pressure) {
        HT3D_LAUNCH(ctx, k_dim_bcs<1>, g, kBlock3, 0, X, B, ky, wN, phc, qyS, _dy, VN, nx, ny, nz);
        HT3D_LAUNCH(ctx, k_dim_bcs<3>, g, kBlock3, 0, X, B, ky, wN, phc, qyS, _dy, VN, nx, ny, nz);
    } else {
        HT3D_LAUNCH(ctx, k_dim_bcs<0>, g, kBlock3, 0, X, B, ky, wN, phc, qyS, _dy, VN, nx, ny, nz);
        HT3D_LAUNCH(ctx, k_dim_bcs<2>, g, kBlock3, 0, X, B, ky, wN, phc, qyS, _dy, VN, nx, ny, nz);
    }
    return HT3D_OK;
}

int ht3d_SetTemperatureBCs(ht3d_ctx* ctx, double* Tc_ex, const double* ky, const double* wN, const double* phc_ex,
                           double qyS, double _dy, double kS, double TS, double TN, double y_plateau, double a2,
                           double b2, double dTdy, double dx, double dy, int sticky_air, double sca_T, double sca_kT,
                           double phi_i, int nx, int ny, int nz) {
    (void)kS; (void)TS; (void)y_plateau; (void)a2; (void)b2; (void)dTdy; (void)dx; (void)dy; (void)sticky_air;
    (void)sca_T; (void)sca_kT; (void)phi_i;
    return ht3d_guard(ctx, [&]() { return dim_bcs(ctx, 0, Tc_ex, ky, wN, phc_ex, qyS, _dy, TN, nx, ny, nz); });
}

int ht3d_SetPressureBCs_dim(ht3d_ctx* ctx, double* Pc_ex, const double* wN, const double* phc_ex, double PS,
                            double PN, double y_plateau, double a2, double b2, double rhof, double g, double dx,
                            double dy, int sticky_air, int nx, int ny, int nz) {
    (void)PS; (void)y_plateau; (void)a2; (void)b2; (void)rhof; (void)g; (void)dx; (void)dy; (void)sticky_air;
    return ht3d_guard(ctx, [&]() { return dim_bcs(ctx, 1, Pc_ex, nullptr, wN, phc_ex, 0.0, 1.0, PN, nx, ny, nz); });
}

int ht3d_PhiRhof(ht3d_ctx* ctx, double* phirhofc, const double* Tc_ex, const double* Pc_ex, const double* phc_ex,
                 double phi_i, double scale_rho, double scale_T, double scale_sigma, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(phirhofc, Tc_ex, Pc_ex, phc_ex), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_phi_rhof, G3(nx, ny, nz), kBlock3, 0, phirhofc, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho,
                    scale_T, scale_sigma, 0, 0, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_PhiRhofOld(ht3d_ctx* ctx, double* phirhofc, const double* Tc0, const double* Pc0, const double* phc_ex,
                    double phi_i, double scale_rho, double scale_T, double scale_sigma, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(phirhofc, Tc0, Pc0, phc_ex), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_phi_rhof, G3(nx, ny, nz), kBlock3, 0, phirhofc, Tc0, Pc0, phc_ex, phi_i, scale_rho, scale_T,
                    scale_sigma, 1, 0, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_PhiDrhodP(ht3d_ctx* ctx, double* phidrhodP, const double* Tc_ex, const double* Pc_ex, const double* phc_ex,
                   double phi_i, double scale_rho, double scale_T, double scale_sigma, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(phidrhodP, Tc_ex, Pc_ex, phc_ex), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_phi_rhof, G3(nx, ny, nz), kBlock3, 0, phidrhodP, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho,
                    scale_T, scale_sigma, 0, 1, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ComputeDarcyFlux(ht3d_ctx* ctx, double* qx, double* qy, double* qz, const double* rhofv, const double* kx,
                          const double* ky, const double* kz, const double* Pf, double g, double _dx, double _dy,
                          double _dz, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(qx, qy, qz, rhofv, kx, ky, kz, Pf), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_darcy_flux, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, qx, qy, qz, rhofv, kx, ky, kz, Pf, g, _dx,
                    _dy, _dz, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_ResidualFluidPressure(ht3d_ctx* ctx, double* F, const double* phc_ex, const double* phirhofc,
                               const double* phirhofc0, const double* PC, const double* qx, const double* qy,
                               const double* qz, double transient, double _dt, double _dx, double _dy, double _dz,
                               int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(F, phc_ex, phirhofc, phirhofc0, PC, qx, qy, qz), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_res_pressure, G3(nx, ny, nz), kBlock3, 0, F, phc_ex, phirhofc, phirhofc0, PC, qx, qy, qz,
                    transient, _dt, _dx, _dy, _dz, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_Init_vel_dim(ht3d_ctx* ctx, double* Vx, double* Vy, double* Vz, const double* qx, const double* qy,
                      const double* qz, const double* rhofv, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Vx, Vy, Vz, qx, qy, qz, rhofv), "null argument");
        DIMS;
        HT3D_LAUNCH(ctx, k_init_vel_dim, G3(nx + 1, ny + 1, nz + 1), kBlock3, 0, Vx, Vy, Vz, qx, qy, qz, rhofv, nx, ny,
                    nz);
        return HT3D_OK;
    });
}

int ht3d_material_law(ht3d_ctx* ctx, int which, const double* a, const double* b, double* out, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(a, out), "null argument");
        HT3D_REQUIRE(which >= 0 && which <= 11 && a && out && n >= 0, "bad argument");
        const unsigned g = (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, ctx->num_sms * 16LL));
        if (n) HT3D_LAUNCH(ctx, k_law_eval, g, 256, 0, out, a, b, which, n);
        return HT3D_OK;
    });
}

}  // extern "C"

// ===========================================================================
// Fused dimensional DYREL solves and the v18 time step.
//
// One launch of k_dim_iter<PRESSURE, MODE> performs one pseudo-iteration of
//   thermal (Dimensional/HydroThermal3D_v18.jl:451-455):
//     SetTemperatureBCs! -> ComputeFlux! -> ResidualTemperatureLinearised! -> DYRELUpdate!
//   Darcy   (v18:510-514):
//     ϕρf -> SetPressureBCs! -> ComputeDarcyFlux! -> ResidualFluidPressure! -> DYRELUpdate!
// reading the snapshot X_in and writing the updated inner cells of X_out.
// The boundary rules are evaluated on the fly for every stencil point
// (bc_value below, the rules of k_dim_bcs in order); the ghost shell of X_out
// is written by k_dim_shell.  Phase codes are read as int8.
// ===========================================================================
#include "dyrel_common.cuh"

void ht3d_weno5_advect_impl(ht3d_ctx* ctx, double* Tc_ex, const double* Vx, const double* Vy, const double* Vz,
                            double dt, double _dx, double _dy, double _dz, const int* bc_type6, const double* bc_val6,
                            int variant, int precision, int nx, int ny, int nz);

namespace {

struct DimBC {
    double VN;        // TN / PN
    double qyS_dy;    // qyS/_dy (thermal bottom flux rule)
    double _dy;
};

// value of ex cell (i,j,k) after the boundary kernel, from snapshot S
template <int PRESSURE>
__device__ __forceinline__ double bc_value(const double* __restrict__ S, const signed char* __restrict__ ph,
                                           const double* __restrict__ wN, const double* __restrict__ ky,
                                           const DimBC& b, int i, int j, int k, int nx, int ny, int nz) {
    const int n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    const int e = EXI(i, j, k);
    double v = S[e];
    const int p = ph[e];
    if (p == 1) v = b.VN;
    const int kmaxx = PRESSURE ? n3 - 2 : n3 - 1;
    if (i == 0 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= kmaxx) v = S[EXI(1, j, k)];
    if (i == n1 - 1 && j >= 1 && j <= n2 - 2 && k >= 1 && k <= kmaxx) v = S[EXI(n1 - 2, j, k)];
    if (j == 0 && i >= 1 && i <= n1 - 2 && k >= 1 && k <= n3 - 2) {
        if (PRESSURE) v = S[EXI(i, 1, k)];
        else v = b.qyS_dy / ky[ix3(i - 1, 0, k - 1, nx, ny + 1)] + S[EXI(i, 1, k)];
    }
    if (p == -1 && j >= 1) {
        const double wn = wN[i + (nx + 2) * k];
        v = (b.VN - (1.0 - wn) * S[EXI(i, j - 1, k)]) / wn;
    }
    if (k == 0 && i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2) v = S[EXI(i, j, 1)];
    if (k == n3 - 1 && i >= 1 && i <= n1 - 2 && j >= 1 && j <= n2 - 2) v = S[EXI(i, j, n3 - 2)];
    return v;
}

// ghost shell of X_out = boundary values of X_in (blockIdx.z: face pair 0 x, 1 y, 2 z)
template <int PRESSURE>
__global__ void k_dim_shell(double* __restrict__ Xout, const double* __restrict__ S, const signed char* __restrict__ ph,
                            const double* __restrict__ wN, const double* __restrict__ ky, DimBC b, int nx, int ny,
                            int nz) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y * blockDim.y + threadIdx.y;
    const int n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    const int face = blockIdx.z >> 1, side = blockIdx.z & 1;
    int i, j, k;
    if (face == 0) { if (a >= n2 || c >= n3) return; i = side ? n1 - 1 : 0; j = a; k = c; }
    else if (face == 1) { if (a >= n1 || c >= n3) return; i = a; j = side ? n2 - 1 : 0; k = c; }
    else { if (a >= n1 || c >= n2) return; i = a; j = c; k = side ? n3 - 1 : 0; }
    Xout[EXI(i, j, k)] = bc_value<PRESSURE>(S, ph, wN, ky, b, i, j, k, nx, ny, nz);
}

struct DimIterArgs {
    const double* Xin;
    double* Xout;
    const signed char* ph;
    const double* wN;
    const double* kx;
    const double* ky;
    const double* kz;
    const double* PC;
    double* F0;
    double* F;
    double* terms;
    // thermal
    const double* T0;
    const double* rC;
    // Darcy
    const double* Tex;     // temperature (ex) for ϕρf
    const double* prf0;    // ϕρf_old
    const double* rfy;     // av_xza(ρfv) on y faces
};

struct DimScal {
    double h1, h2, dtau, _dx, _dy, _dz, _dt, transient, Qt, g;
    double phi_i, s_rho, s_T, s_sigma;
};

template <int PRESSURE, int MODE>
__global__ void __launch_bounds__(CX_* CY_* CZ_) k_dim_iter(DimIterArgs A, DimScal s, DimBC b, int nx, int ny, int nz) {
    const int i = blockIdx.x * CX_ + threadIdx.x;
    const int j = blockIdx.y * CY_ + threadIdx.y;
    const int k = blockIdx.z * CZ_ + threadIdx.z;
    if (i >= nx || j >= ny || k >= nz) return;
    const int I = i + 1, J = j + 1, K = k + 1;
    const int c = CI(i, j, k);
    auto X = [&](int ii, int jj, int kk) {
        return bc_value<PRESSURE>(A.Xin, A.ph, A.wN, A.ky, b, ii, jj, kk, nx, ny, nz);
    };
    const double xc = X(I, J, K);
    const double xw = X(I - 1, J, K), xe = X(I + 1, J, K);
    const double xs = X(I, J - 1, K), xn = X(I, J + 1, K);
    const double xb = X(I, J, K - 1), xf = X(I, J, K + 1);
    const int fx = ix3(i, j, k, nx + 1, ny), fy = ix3(i, j, k, nx, ny + 1);
    const double qW = -A.kx[fx] * (s._dx * (xc - xw));
    const double qE = -A.kx[fx + 1] * (s._dx * (xe - xc));
    const double qB = -A.kz[c] * (s._dz * (xc - xb));
    const double qF = -A.kz[c + nx * ny] * (s._dz * (xf - xc));
    double qS, qN;
    if (PRESSURE) {
        qS = -A.ky[fy] * (s._dy * (xc - xs) - s.g * A.rfy[fy]);
        qN = -A.ky[fy + nx] * (s._dy * (xn - xc) - s.g * A.rfy[fy + nx]);
    } else {
        qS = -A.ky[fy] * (s._dy * (xc - xs));
        qN = -A.ky[fy + nx] * (s._dy * (xn - xc));
    }
    const int e = EXI(I, J, K);
    const int p = A.ph[e];
    double f = 0.;
    if (p != 1 && p != -1) {
        if (PRESSURE) {
            // ϕρf from the pre-boundary-kernel pressure (the reference runs ϕρf first)
            const double Tc = A.Tex[e] * s.s_T - 273.15;
            const double Pc = A.Xin[e] * s.s_sigma;
            const double prf = law_phi((double)p, s.phi_i) * law_rhof_C(Tc, Pc) / s.s_rho;
            f = s.transient * s._dt * (prf - A.prf0[c]);
        } else {
            double Q = 0.;
            if (p == 3) Q = s.Qt;
            f = s.transient * A.rC[c] * s._dt * (xc - A.T0[c]);
            f += (qE - qW) * s._dx;
            f += (qN - qS) * s._dy;
            f += (qF - qB) * s._dz;
            f -= s.transient * Q;
            f /= A.PC[c];
        }
        if (PRESSURE) {
            f += (qE - qW) * s._dx;
            f += (qN - qS) * s._dy;
            f += (qF - qB) * s._dz;
            f /= A.PC[c];
        }
    }
    const double f0 = s.h1 * A.F0[c] + s.h2 * f;
    A.F0[c] = f0;
    A.Xout[e] = xc - s.dtau * f0;
    if (MODE == MODE_CHECK) {
        const double fit = A.F[c];
        const double d = s.dtau * f0;
        const int n = nx * ny * nz;
        A.terms[c] = fabs(f * A.PC[c]);
        A.terms[c + n] = -d * (f - fit);
        A.terms[c + 2 * n] = d * d;
    }
    if (MODE >= MODE_STOREF) A.F[c] = f;
}

__global__ void k_pluton(double* T, const double* __restrict__ phc, double Tp, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        if (ph_eq(phc[t], 3.0)) T[t] = Tp;
}
__global__ void k_phase8(signed char* out, const double* __restrict__ phc, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = (signed char)phc[t];
}
__global__ void k_av_xza(double* out, const double* __restrict__ rfv, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny + 1 || k >= nz) return;
    out[ix3(i, j, k, nx, ny + 1)] =
        (rfv[VXI(i, j, k)] + rfv[VXI(i + 1, j, k)] + rfv[VXI(i, j, k + 1)] + rfv[VXI(i + 1, j, k + 1)]) * 0.25;
}
__global__ void k_inn_copy(double* A, const double* __restrict__ B, int nx, int ny, int nz) {
    for_cells_z(nx, ny, nz, [&](int i, int j, int k) { A[CI(i, j, k)] = B[EXI(i + 1, j + 1, k + 1)]; });
}
__global__ void k_gersh(double* G, double* D, const double* __restrict__ rC, const double* __restrict__ kx,
                        const double* __restrict__ ky, const double* __restrict__ kz, double transient, double dt,
                        double dx, double dy, double dz, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const double kW = kx[ix3(i, j, k, nx + 1, ny)], kE = kx[ix3(i + 1, j, k, nx + 1, ny)];
    const double kS = ky[ix3(i, j, k, nx, ny + 1)], kN = ky[ix3(i, j + 1, k, nx, ny + 1)];
    const double kB = kz[CI(i, j, k)], kF = kz[CI(i, j, k + 1)], rhoC = rC[CI(i, j, k)];
    const double diag = ((kB / dz + kF / dz) / dz + (kN / dy + kS / dy) / dy + (kE / dx + kW / dx) / dx + rhoC * transient / dt);
    double g = fabs(kE / (dx * dx)) + fabs(kW / (dx * dx)) + fabs(kN / (dy * dy)) + fabs(kS / (dy * dy)) +
               fabs(kB / (dz * dz)) + fabs(kF / (dz * dz)) + fabs(diag);
    D[CI(i, j, k)] = diag;
    G[CI(i, j, k)] = g / diag;
}

struct DimWork {
    double *X2, *kv, *dumc, *kx, *ky, *kz, *rC, *PC, *G, *F, *F0, *T0, *P0, *rfy, *terms, *prf0;
    const double* Tex;  // temperature (ex) read by the Darcy iteration
    signed char* ph;
};

// DYREL loop of Dimensional/HydroThermal3D_v18.jl:443-477 / :504-537 on the fused kernel
template <int PRESSURE>
int dim_dyrel(ht3d_ctx* ctx, double* X, DimWork& W, const double* wN, DimScal s, DimBC b, double lmax,
              const ht3d_dyrel_params* prm, ht3d_dyrel_stats* st, int nx, int ny, int nz) {
    const long long n = (long long)nx * ny * nz;
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    HT3D_REQUIRE(prm->nitout >= 1 && prm->nitmax >= 1, "nitout and nitmax must be >= 1");
    DyrelState S;
    dyrel_init_params(prm, lmax, S);
    HT3D_CUDA(cudaMemsetAsync(W.F, 0, sizeof(double) * n, ctx->stream));
    HT3D_CUDA(cudaMemsetAsync(W.F0, 0, sizeof(double) * n, ctx->stream));
    // both buffers start identical so cells no rule writes stay equal
    HT3D_CUDA(cudaMemcpyAsync(W.X2, X, sizeof(double) * nex, cudaMemcpyDeviceToDevice, ctx->stream));
    const dim3 blk(CX_, CY_, CZ_), grd((nx + CX_ - 1) / CX_, (ny + CY_ - 1) / CY_, (nz + CZ_ - 1) / CZ_);
    const int nm = std::max(nx, std::max(ny, nz)) + 2;
    const dim3 sb(32, 8, 1), sg((nm + 31) / 32, (nm + 7) / 8, 6);
    DimIterArgs A;
    A.ph = W.ph; A.wN = wN; A.kx = W.kx; A.ky = W.ky; A.kz = W.kz; A.PC = W.PC; A.F0 = W.F0; A.F = W.F;
    A.terms = W.terms; A.T0 = W.T0; A.rC = W.rC; A.Tex = W.Tex; A.prf0 = W.prf0; A.rfy = W.rfy;
    double* cur = X;
    double* nxt = W.X2;
    DyrelCheck C;
    int it_done = 0;
    for (int iter = 1; iter <= prm->nitmax; ++iter) {
        const bool chk = is_check(iter, prm->nitout);
        const bool storef = !chk && (iter == prm->nitmax || is_check(iter + 1, prm->nitout));
        s.h1 = S.h1; s.h2 = S.h2; s.dtau = S.dtau;
        A.Xin = cur; A.Xout = nxt;
        if (chk) HT3D_LAUNCH(ctx, (k_dim_iter<PRESSURE, MODE_CHECK>), grd, blk, 0, A, s, b, nx, ny, nz);
        else if (storef) HT3D_LAUNCH(ctx, (k_dim_iter<PRESSURE, MODE_STOREF>), grd, blk, 0, A, s, b, nx, ny, nz);
        else HT3D_LAUNCH(ctx, (k_dim_iter<PRESSURE, MODE_PLAIN>), grd, blk, 0, A, s, b, nx, ny, nz);
        HT3D_LAUNCH(ctx, k_dim_shell<PRESSURE>, sg, sb, 0, nxt, cur, W.ph, wN, W.ky, b, nx, ny, nz);
        std::swap(cur, nxt);
        it_done = iter;
        if (chk) {
            tree_sum3(ctx, W.terms, n, W.terms + 3 * n);
            if (C.update(S, prm, ctx->h_result[0], ctx->h_result[1], ctx->h_result[2], (double)n, iter, true)) break;
        }
    }
    if (cur != X) HT3D_CUDA(cudaMemcpyAsync(X, cur, sizeof(double) * nex, cudaMemcpyDeviceToDevice, ctx->stream));
    C.fill(st, S, it_done);
    return C.status;
}

}  // namespace

extern "C" int ht3d_sizeof_v18_params(void) { return (int)sizeof(ht3d_v18_params); }

extern "C" int ht3d_step_v18(ht3d_ctx* ctx, double* Tc_ex, double* Pc_ex, const double* phc_ex, const double* phv,
                             const double* wN, const double* kmul_v, double* Vx, double* Vy, double* Vz,
                             ht3d_v18_params* p, ht3d_dyrel_stats* st_T, ht3d_dyrel_stats* st_P, int nx, int ny,
                             int nz) {
    return ht3d_guard(ctx, [&]() {
        NvtxRange range("ht3d step_v18");
        ht3d_check_dims(nx, ny, nz, 3);
        HT3D_REQUIRE(Tc_ex && Pc_ex && phc_ex && phv && wN && Vx && Vy && Vz && p, "null argument");
        HT3D_REQUIRE(p->dt > 0.0, "dt must be positive");
        const long long n = (long long)nx * ny * nz, nv = (long long)(nx + 1) * (ny + 1) * (nz + 1),
                        nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
        const long long nfx = (long long)(nx + 1) * ny * nz, nfy = (long long)nx * (ny + 1) * nz,
                        nfz = (long long)nx * ny * (nz + 1);
        DimWork W;
        W.Tex = Tc_ex;
        W.prf0 = nullptr;
        W.X2 = (double*)ht3d_scratch(ctx, SLOT_X2, sizeof(double) * nex);
        W.kv = (double*)ht3d_scratch(ctx, SLOT_AUX0, sizeof(double) * nv);
        W.dumc = (double*)ht3d_scratch(ctx, SLOT_AUX1, sizeof(double) * n);
        W.kx = (double*)ht3d_scratch(ctx, SLOT_STEP_KX, sizeof(double) * nfx);
        W.ky = (double*)ht3d_scratch(ctx, SLOT_STEP_KY, sizeof(double) * nfy);
        W.kz = (double*)ht3d_scratch(ctx, SLOT_STEP_KZ, sizeof(double) * nfz);
        W.rC = (double*)ht3d_scratch(ctx, SLOT_STEP_R, sizeof(double) * n);
        W.PC = (double*)ht3d_scratch(ctx, SLOT_PC, sizeof(double) * n);
        W.G = (double*)ht3d_scratch(ctx, SLOT_G, sizeof(double) * n);
        W.F = (double*)ht3d_scratch(ctx, SLOT_STEP_F, sizeof(double) * n);
        W.F0 = (double*)ht3d_scratch(ctx, SLOT_STEP_F0, sizeof(double) * n);
        W.T0 = (double*)ht3d_scratch(ctx, SLOT_WENO_T0, sizeof(double) * n);
        W.P0 = (double*)ht3d_scratch(ctx, SLOT_WENO_T2, sizeof(double) * n);
        W.rfy = (double*)ht3d_scratch(ctx, SLOT_STEP_TY, sizeof(double) * nfy);
        W.terms = (double*)ht3d_scratch(ctx, SLOT_PARTIALS, sizeof(double) * (3 * n + 6 * ((n + 1023) / 1024 + 1)));
        W.ph = (signed char*)ht3d_scratch(ctx, SLOT_AUX2, nex);
        const double dx = p->dx, dy = p->dy, dz = p->dz, _dx = 1.0 / dx, _dy = 1.0 / dy, _dz = 1.0 / dz;
        const double dt = p->dt, _dt = 1.0 / dt, transient = p->it == 0 ? 0.0 : 1.0;
        const dim3 gv = grid3(nx + 1, ny + 1, nz + 1, kBlock3), gc = grid3(nx, ny, nz, kBlock3);
        const unsigned g1 = (unsigned)std::max<long long>(1, std::min<long long>((nex + 255) / 256, ctx->num_sms * 16LL));
        if (p->it == 1) HT3D_LAUNCH(ctx, k_pluton, g1, 256, 0, Tc_ex, phc_ex, p->T_pluton, nex);
        HT3D_LAUNCH(ctx, k_phase8, g1, 256, 0, W.ph, phc_ex, nex);
        HT3D_LAUNCH(ctx, k_inn_copy, grid3z(nx, ny, nz), kBlock3, 0, W.T0, Tc_ex, nx, ny, nz);
        HT3D_LAUNCH(ctx, k_inn_copy, grid3z(nx, ny, nz), kBlock3, 0, W.P0, Pc_ex, nx, ny, nz);
        HT3D_CUDA(cudaMemsetAsync(W.rC, 0, sizeof(double) * n, ctx->stream));
        DimScal s{};
        s._dx = _dx; s._dy = _dy; s._dz = _dz; s._dt = _dt; s.transient = transient; s.Qt = p->Qt; s.g = p->g;
        s.phi_i = p->phi_i; s.s_rho = p->sc_rho; s.s_T = p->sc_T; s.s_sigma = p->sc_sigma;
        auto smooth = [&]() {
            HT3D_LAUNCH(ctx, k_smooth_v2c, gc, kBlock3, 0, W.dumc, W.kv, nx, ny, nz);
            HT3D_LAUNCH(ctx, k_smooth_c2v, grid3(nx - 1, ny - 1, nz - 1, kBlock3), kBlock3, 0, W.kv, W.dumc, nx, ny, nz);
            HT3D_LAUNCH(ctx, k_init_conductivity, gv, kBlock3, 0, W.kx, W.ky, W.kz, W.kv, nx, ny, nz);
        };
        int st = HT3D_OK;
        if (p->thermal) {
            HT3D_LAUNCH(ctx, k_thermal_conductivity, gv, kBlock3, 0, W.kv, Tc_ex, phv, p->phi_i, p->sc_kt, p->sc_T, nx,
                        ny, nz);
            smooth();
            HT3D_LAUNCH(ctx, k_rhoC_eff, gc, kBlock3, 0, W.rC, Tc_ex, Pc_ex, phc_ex, p->phi_i, p->sc_T, p->sc_sigma,
                        p->sc_C, p->sc_rho, nx, ny, nz);
            HT3D_LAUNCH(ctx, k_gersh, gc, kBlock3, 0, W.G, W.PC, W.rC, W.kx, W.ky, W.kz, transient, dt, dx, dy, dz, nx,
                        ny, nz);
            DimBC b{p->Ttop, p->qyS / _dy, _dy};
            const double lmax = ht3d_reduce_device(ctx, W.G, n, RED_MAX, nullptr);
            st = dim_dyrel<0>(ctx, Tc_ex, W, wN, s, b, lmax, &p->thermal_dyrel, st_T, nx, ny, nz);
            if (st) return st;
        }
        if (p->hydro) {
            HT3D_LAUNCH(ctx, k_hydro_conductivity, gv, kBlock3, 0, W.kv, Tc_ex, Pc_ex, phv, p->ymin, dy, p->k_fact,
                        p->delta, p->sc_sigma, p->sc_T, p->sc_L, p->sc_t, p->sc_eta, 1, kmul_v, nx, ny, nz);
            smooth();
            HT3D_LAUNCH(ctx, k_phi_rhof, gc, kBlock3, 0, W.rC, Tc_ex, Pc_ex, phc_ex, p->phi_i, p->sc_rho, p->sc_T,
                        p->sc_sigma, 0, 1, nx, ny, nz);
            HT3D_LAUNCH(ctx, k_gersh, gc, kBlock3, 0, W.G, W.PC, W.rC, W.kx, W.ky, W.kz, transient, dt, dx, dy, dz, nx,
                        ny, nz);
            const double lmax = ht3d_reduce_device(ctx, W.G, n, RED_MAX, nullptr);
            // the reference reuses the Gershgorin array (Xc0) for ϕρf_old (v18:500)
            HT3D_LAUNCH(ctx, k_phi_rhof, gc, kBlock3, 0, W.G, W.T0, W.P0, phc_ex, p->phi_i, p->sc_rho, p->sc_T,
                        p->sc_sigma, 1, 0, nx, ny, nz);
            W.prf0 = W.G;
            HT3D_LAUNCH(ctx, k_fluid_density, gv, kBlock3, 0, W.kv, Tc_ex, Pc_ex, phv, p->sc_sigma, p->sc_T, p->sc_rho,
                        nx, ny, nz);
            HT3D_LAUNCH(ctx, k_av_xza, grid3(nx, ny + 1, nz, kBlock3), kBlock3, 0, W.rfy, W.kv, nx, ny, nz);
            DimBC b{p->Ptop, 0.0, _dy};
            st = dim_dyrel<1>(ctx, Pc_ex, W, wN, s, b, lmax, &p->darcy_dyrel, st_P, nx, ny, nz);
            if (st) return st;
        }
        // velocity (v18:543-548)
        HT3D_LAUNCH(ctx, k_hydro_conductivity, gv, kBlock3, 0, W.kv, Tc_ex, Pc_ex, phv, p->ymin, dy, p->k_fact, p->delta,
                    p->sc_sigma, p->sc_T, p->sc_L, p->sc_t, p->sc_eta, 2, kmul_v, nx, ny, nz);
        smooth();
        HT3D_LAUNCH(ctx, k_fluid_density, gv, kBlock3, 0, W.kv, Tc_ex, Pc_ex, phv, p->sc_sigma, p->sc_T, p->sc_rho, nx,
                    ny, nz);
        HT3D_LAUNCH(ctx, k_darcy_flux, gv, kBlock3, 0, Vx, Vy, Vz, W.kv, W.kx, W.ky, W.kz, Pc_ex, p->g, _dx, _dy, _dz,
                    nx, ny, nz);
        p->n_adv = 0;
        if (p->it > 0) {
            p->time += dt;
            if (p->advection) {
                double* dres = (double*)ht3d_scratch(ctx, SLOT_RESULT, sizeof(double) * 64);
                ht3d_reduce_device(ctx, Vx, nfx, RED_MAX_ABS, dres + 8);
                ht3d_reduce_device(ctx, Vy, nfy, RED_MAX_ABS, dres + 9);
                ht3d_reduce_device(ctx, Vz, nfz, RED_MAX_ABS, dres + 10);
                ht3d_fetch_results(ctx, dres + 8, 3);
                const double vmax = std::max(std::max(ctx->h_result[0], ctx->h_result[1]), ctx->h_result[2]);
                const double dt_adv = p->C_adv * 1.0 / 6.1 * std::min(std::min(dx, dy), dz) / vmax;
                const int bt[6] = {0, 0, 1, 1, 0, 0};
                const double bv[6] = {0.0, 0.0, p->Tbot, p->Ttop, 0.0, 0.0};
                if (!p->dt_constant) {
                    p->dt = dt_adv;
                    ht3d_weno5_advect_impl(ctx, Tc_ex, Vx, Vy, Vz, p->dt, _dx, _dy, _dz, bt, bv, p->weno_variant,
                                           HT3D_FP64, nx, ny, nz);
                    p->n_adv = 1;
                } else {
                    const double na = std::ceil(dt / dt_adv);
                    HT3D_REQUIRE(na >= 1.0 && na <= 32767.0, "advection sub-step count out of Int16 range");
                    const int nt_adv = (int)na;
                    const double dt_adv1 = dt / nt_adv;
                    for (int ia = 0; ia < nt_adv; ++ia)
                        ht3d_weno5_advect_impl(ctx, Tc_ex, Vx, Vy, Vz, dt_adv1, _dx, _dy, _dz, bt, bv,
                                               p->weno_variant, HT3D_FP64, nx, ny, nz);
                    p->n_adv = nt_adv;
                }
            }
        }
        return HT3D_OK;
    });
}


// ---------------------------------------------------------------------------
// SetInitialConditions_Khaled (Dimensional/HydroThermal3D_v18.jl:59-129).
// Every value is a pure function of the point's coordinates, so the
// reference's sequence of whole-array statements (phase masks overriding one
// another; T, P profiles followed by the x-, y- and z-ghost statements and the
// air override) is evaluated per point in that order.
// ---------------------------------------------------------------------------
namespace {

struct KhaledArgs {
    ht3d_khaled_geom g;
    double Tbot, Ttop, Pbot, Ptop, xmin, ymin, zmin, xmax, ymax, zmax, L;
    double dx, dy, dz, cos_t, sin_t;
};

// element i of Julia's LinRange(a, b, n): (1 - t) a + t b, t = i / (n - 1)
__device__ __forceinline__ double linrange(double a, double b, long long n, long long i) {
    const double t = (double)i / (double)(n - 1);
    return (1.0 - t) * a + t * b;
}

// Topography (v18.jl:43-57)
__device__ __forceinline__ double topography(double x, double y_plateau, double a2, double b2) {
    const double xW = -b2 / a2;
    const double xE = (y_plateau - b2) / a2;
    if (x <= xW) return 0.0;
    if (x >= xE) return y_plateau;
    return a2 * x + b2;
}

__device__ double khaled_phase(double x, double y, double z, double y0, const KhaledArgs& A) {
    double ph = 0.0;  // crust
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const double* c = A.g.fault[f];
        if (y < (x * c[0] + c[1]) && y > (x * c[2] + c[3]) && y > (x * c[4] + c[5])) ph = 2.0;
    }
    const double a = 1e3 / A.L, b = 10e3 / A.L, cz = 500e3 / A.L, z0 = A.zmax / 2;
    const double x0 = 53057.07323 / A.L, yp = -8992.45195 / A.L;
    const double u = ((x - x0) * A.cos_t - (y - yp) * A.sin_t) / a;
    const double v = ((x - x0) * A.sin_t + (y - yp) * A.cos_t) / b;
    const double w = (z - z0) / cz;
    if (u * u + v * v + w * w < 1) ph = 3.0;
    const double tiny = 1e-9;
    if (y > (y0 - tiny)) ph = 1.0;  // air
    return ph;
}

__global__ void k_khaled_vertices(double* __restrict__ phv, KhaledArgs A, int nx, int ny, int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > nx || j > ny || k > nz) return;
    const double x = linrange(A.xmin, A.xmax, nx + 1, i), y = linrange(A.ymin, A.ymax, ny + 1, j),
                 z = linrange(A.zmin, A.zmax, nz + 1, k);
    const double y0 = topography(x, A.g.y_plateau, A.g.surf_a1, A.g.surf_b1);
    phv[i + (long long)(nx + 1) * (j + (long long)(ny + 1) * k)] = khaled_phase(x, y, z, y0, A);
}

__device__ double khaled_field(double Vtop, double Vbot, int i, int j, const KhaledArgs& A, int n1, int n2) {
    const double y_bot = -30e3 / A.L;
    auto xce = [&](int ii) { return linrange(A.xmin - A.dx / 2, A.xmax + A.dx / 2, n1, ii); };
    auto yce = [&](int jj) { return linrange(A.ymin - A.dy / 2, A.ymax + A.dy / 2, n2, jj); };
    auto profile = [&](int ii, int jj) {
        const double y0 = topography(xce(ii), A.g.y_plateau, A.g.surf_a1, A.g.surf_b1);
        const double dVdy = (Vtop - Vbot) / (y0 - y_bot);
        return Vtop + dVdy * (yce(jj) - y0);
    };
    auto vx = [&](int ii, int jj) { return profile(ii == 0 ? 1 : (ii == n1 - 1 ? n1 - 2 : ii), jj); };
    double v;
    if (j == 0) v = 2 * Vbot - vx(i, 1);
    else if (j == n2 - 1) v = 2 * Vtop - vx(i, n2 - 2);
    else v = vx(i, j);
    const double x = xce(i), y = yce(j);
    if ((y > 0 && (y > (x * A.g.surf_a1 + A.g.surf_b1))) || y > A.g.y_plateau) v = Vtop;
    return v;
}

__global__ void k_khaled_cells(double* __restrict__ phc, double* __restrict__ T, double* __restrict__ P, KhaledArgs A,
                               int nx, int ny, int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    if (i >= n1 || j >= n2 || k >= n3) return;
    const long long e = i + (long long)n1 * (j + (long long)n2 * k);
    const double x = linrange(A.xmin - A.dx / 2, A.xmax + A.dx / 2, n1, i);
    const double y = linrange(A.ymin - A.dy / 2, A.ymax + A.dy / 2, n2, j);
    const double z = linrange(A.zmin - A.dz / 2, A.zmax + A.dz / 2, n3, k);
    const double y0 = topography(x, A.g.y_plateau, A.g.surf_a1, A.g.surf_b1);
    phc[e] = khaled_phase(x, y, z, y0, A);
    T[e] = khaled_field(A.Ttop, A.Tbot, i, j, A, n1, n2);
    P[e] = khaled_field(A.Ptop, A.Pbot, i, j, A, n1, n2);
}

}  // namespace

extern "C" int ht3d_SetInitialConditions_Khaled(ht3d_ctx* ctx, double* phc_ex, double* phv, double* wN,
                                                const ht3d_khaled_geom* geom, double* Tc_ex, double* Pc_ex,
                                                double Tbot, double Ttop, double Pbot, double Ptop, double xmin,
                                                double ymin, double zmin, double xmax, double ymax, double zmax,
                                                double L, int nx, int ny, int nz) {
    (void)wN;
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(phc_ex, phv, geom, Tc_ex, Pc_ex), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        HT3D_REQUIRE(xmax > xmin && ymax > ymin && zmax > zmin && L > 0, "empty domain");
        KhaledArgs A;
        A.g = *geom;
        A.Tbot = Tbot; A.Ttop = Ttop; A.Pbot = Pbot; A.Ptop = Ptop;
        A.xmin = xmin; A.ymin = ymin; A.zmin = zmin; A.xmax = xmax; A.ymax = ymax; A.zmax = zmax; A.L = L;
        A.dx = (xmax - xmin) / nx;
        A.dy = (ymax - ymin) / ny;
        A.dz = (zmax - zmin) / nz;
        const double t_ta = 60 * (M_PI / 180);  // the pluton's rotation, evaluated on the host like the oracle's
        A.cos_t = cos(t_ta);
        A.sin_t = sin(t_ta);
        const dim3 b(32, 8, 1);
        HT3D_LAUNCH(ctx, k_khaled_vertices, dim3((nx + 1 + 31) / 32, (ny + 1 + 7) / 8, nz + 1), b, 0, phv, A, nx, ny, nz);
        HT3D_LAUNCH(ctx, k_khaled_cells, dim3((nx + 2 + 31) / 32, (ny + 2 + 7) / 8, nz + 2), b, 0, phc_ex, Tc_ex, Pc_ex,
                    A, nx, ny, nz);
        return HT3D_OK;
    });
}
