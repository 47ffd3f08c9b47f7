// Time-step driver of the dimensionless Horton-Rogers-Lapwood model
// (Dimensionless/HydroThermal3D_Alban_v6.jl:322-464 with the DYREL solver of
// Dimensional/HydroThermal3D_v18.jl:432-537 and the adaptive dt of
// Dimensionless/HydroThermal3D_v7.jl:220).
#include "ht3d_internal.cuh"

int ht3d_dyrel_solve_fp64(ht3d_ctx* ctx, double* X, const double* R, const double* kx, const double* ky,
                          const double* kz, double cX, double dx, double dy, double dz, const int* bc_type6,
                          const double* bc_val6, const ht3d_dyrel_params* prm, int n_iter_fixed, double* F, double* F0,
                          ht3d_dyrel_stats* st, int nx, int ny, int nz);
int ht3d_dyrel_solve_mixed(ht3d_ctx* ctx, double* X, const double* R, const double* kx, const double* ky,
                           const double* kz, double cX, double dx, double dy, double dz, const int* bc_type6,
                           const double* bc_val6, const ht3d_dyrel_params* prm, int n_iter_fixed, double* F,
                           double* F0, ht3d_dyrel_stats* st, int nx, int ny, int nz);
void ht3d_weno5_advect_impl(ht3d_ctx* ctx, double* Tc_ex, const double* Vx, const double* Vy, const double* Vz,
                            double dt, double _dx, double _dy, double _dz, const int* bc_type6, const double* bc_val6,
                            int variant, int precision, int nx, int ny, int nz);

#include "step_kernels.cuh"

int ht3d_step_hrl_impl(ht3d_ctx* ctx, double* Tc_ex, double* Pc_ex, const double* ktv, const double* kfv, double* Vx,
                       double* Vy, double* Vz, ht3d_hrl_params* p, ht3d_dyrel_stats* st_thermal,
                       ht3d_dyrel_stats* st_darcy, int precision, int nx, int ny, int nz) {
    NvtxRange range("ht3d step_hrl");
    ht3d_check_dims(nx, ny, nz, 1);
    HT3D_REQUIRE(Tc_ex && Pc_ex && ktv && kfv && Vx && Vy && Vz && p, "null argument");
    HT3D_REQUIRE(precision == HT3D_FP64 || precision == HT3D_MIXED, "unknown precision");
    HT3D_REQUIRE(p->dt > 0.0, "dt must be positive");
    const long long n = (long long)nx * ny * nz;
    const long long nfx = (long long)(nx + 1) * ny * nz, nfy = (long long)nx * (ny + 1) * nz,
                    nfz = (long long)nx * ny * (nz + 1);
    double* R = (double*)ht3d_scratch(ctx, SLOT_STEP_R, sizeof(double) * n);
    double* F = (double*)ht3d_scratch(ctx, SLOT_STEP_F, sizeof(double) * n);
    double* F0 = (double*)ht3d_scratch(ctx, SLOT_STEP_F0, sizeof(double) * n);
    double* Ty = (double*)ht3d_scratch(ctx, SLOT_STEP_TY, sizeof(double) * nfy);
    double* kx = (double*)ht3d_scratch(ctx, SLOT_STEP_KX, sizeof(double) * nfx);
    double* ky = (double*)ht3d_scratch(ctx, SLOT_STEP_KY, sizeof(double) * nfy);
    double* kz = (double*)ht3d_scratch(ctx, SLOT_STEP_KZ, sizeof(double) * nfz);
    const double _dx = 1.0 / p->dx, _dy = 1.0 / p->dy, _dz = 1.0 / p->dz, _dt = 1.0 / p->dt;
    const dim3 gv = grid3(nx + 1, ny + 1, nz + 1, kBlock3), gc = grid3(nx, ny, nz, kBlock3);
    auto solve = precision == HT3D_FP64 ? ht3d_dyrel_solve_fp64 : ht3d_dyrel_solve_mixed;
    // thermal
    HT3D_LAUNCH(ctx, k_step_init_thermal, gv, kBlock3, 0, R, kx, ky, kz, Tc_ex, ktv, _dt, nx, ny, nz);
    int s = solve(ctx, Tc_ex, R, kx, ky, kz, _dt, p->dx, p->dy, p->dz, p->thermal_bc, p->thermal_val, &p->thermal,
                  0, F, F0, st_thermal, nx, ny, nz);
    if (s) return s;
    // Darcy
    HT3D_LAUNCH(ctx, k_step_init_darcy, gv, kBlock3, 0, Ty, kx, ky, kz, Tc_ex, kfv, p->kill_ns, nx, ny, nz);
    HT3D_LAUNCH(ctx, k_step_rp, gc, kBlock3, 0, R, ky, Ty, p->Ra, _dy, nx, ny, nz);
    s = solve(ctx, Pc_ex, R, kx, ky, kz, 0.0, p->dx, p->dy, p->dz, p->darcy_bc, p->darcy_val, &p->darcy, 0, F, F0,
              st_darcy, nx, ny, nz);
    if (s) return s;
    // velocity and advection
    HT3D_LAUNCH(ctx, k_step_vel, gv, kBlock3, 0, Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty, p->Ra, _dx, _dy, _dz, nx, ny, nz);
    if (p->advection)
        ht3d_weno5_advect_impl(ctx, Tc_ex, Vx, Vy, Vz, p->dt, _dx, _dy, _dz, p->weno_bc, p->weno_val,
                               p->weno_variant, precision, nx, ny, nz);
    if (p->dt_adapt) {
        double* dres = (double*)ht3d_scratch(ctx, SLOT_RESULT, sizeof(double) * 64);
        ht3d_reduce_device(ctx, Vx, nfx, RED_MAX_ABS, dres + 8);
        ht3d_reduce_device(ctx, Vy, nfy, RED_MAX_ABS, dres + 9);
        ht3d_reduce_device(ctx, Vz, nfz, RED_MAX_ABS, dres + 10);
        ht3d_fetch_results(ctx, dres + 8, 3);
        const double vmax = std::max(std::max(ctx->h_result[0], ctx->h_result[1]), ctx->h_result[2]);
        p->dt = p->dt_fact * 1.0 / 6.1 * std::min(std::min(p->dx, p->dy), p->dz) / vmax;
        if (p->dt_max > 0.0 && p->dt > p->dt_max) p->dt = p->dt_max;
    }
    return HT3D_OK;
}

extern "C" int ht3d_step_hrl(ht3d_ctx* ctx, double* Tc_ex, double* Pc_ex, const double* ktv, const double* kfv,
                             double* Vx, double* Vy, double* Vz, ht3d_hrl_params* p, ht3d_dyrel_stats* st_thermal,
                             ht3d_dyrel_stats* st_darcy, int precision, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        return ht3d_step_hrl_impl(ctx, Tc_ex, Pc_ex, ktv, kfv, Vx, Vy, Vz, p, st_thermal, st_darcy, precision, nx, ny,
                                  nz);
    });
}
