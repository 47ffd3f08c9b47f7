// Plain FP64 DYREL solver.  Compiled with -fmad=false: every pseudo-iteration
// rounds exactly like the reference's separate kernels (no FMA contraction,
// F divided by PC), so the solver differs from the reference only through the
// summation order of its norm and Rayleigh-quotient reductions.
#include "dyrel_common.cuh"

int ht3d_dyrel_solve_fp64(ht3d_ctx* ctx, double* X, const double* R, const double* kx, const double* ky,
                          const double* kz, double cX, double dx, double dy, double dz, const int* bc_type6,
                          const double* bc_val6, const ht3d_dyrel_params* prm, int n_iter_fixed, double* F, double* F0,
                          ht3d_dyrel_stats* st, int nx, int ny, int nz) {
    NvtxRange range("ht3d DYREL solve (FP64)");
    const long long n = (long long)nx * ny * nz;
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    double* PC = (double*)ht3d_scratch(ctx, SLOT_PC, sizeof(double) * n);
    double* X2 = (double*)ht3d_scratch(ctx, SLOT_X2, sizeof(double) * nex);
    IterLaunch L = iter_launch(ctx, nx, ny, nz);
    const long long nsetup = (long long)((nx + 31) / 32) * ((ny + 7) / 8) * nz;
    // per-cell check terms (3n) followed by tree-pass work space
    const long long nwork = 3 * n + 6 * ((n + 1023) / 1024 + 1);
    double* parts = (double*)ht3d_scratch(ctx, SLOT_PARTIALS, sizeof(double) * std::max(nwork, nsetup));
    double* dres = (double*)ht3d_scratch(ctx, SLOT_RESULT, sizeof(double) * 64);

    BC6<double> bc;
    for (int f = 0; f < 6; ++f) {
        HT3D_REQUIRE(bc_type6[f] == HT3D_BC_NEUMANN || bc_type6[f] == HT3D_BC_DIRICHLET, "face BC type must be 0 or 1");
        bc.dir[f] = bc_type6[f];
        bc.val2[f] = 2.0 * bc_val6[f];
    }
    // Gershgorin lambda_max and preconditioner
    {
        dim3 b(32, 8, 1), g((nx + 31) / 32, (ny + 7) / 8, nz);
        const double transient = cX != 0.0 ? 1.0 : 0.0, dt = cX != 0.0 ? 1.0 / cX : 1.0;
        HT3D_LAUNCH(ctx, k_dyrel_setup<0>, g, b, 0, kx, ky, kz, 1.0, transient, dt, dx, dy, dz, nx, ny, nz, PC, parts);
        HT3D_LAUNCH(ctx, (k_reduce_partials<RED_MAX, 1>), 1, 1024, 0, parts, (int)(g.x * g.y * g.z), dres);
        ht3d_fetch_results(ctx, dres, 1);
    }
    DyrelState S;
    dyrel_init_params(prm, ctx->h_result[0], S);
    HT3D_CUDA(cudaMemsetAsync(F, 0, sizeof(double) * n, ctx->stream));
    HT3D_CUDA(cudaMemsetAsync(F0, 0, sizeof(double) * n, ctx->stream));

    DyrelScal sc;
    sc.cX = cX;
    sc._dx = 1.0 / dx;
    sc._dy = 1.0 / dy;
    sc._dz = 1.0 / dz;
    double* cur = X;
    double* nxt = X2;
    DyrelCheck C;
    int it_done = 0;
    const int nmax = n_iter_fixed > 0 ? n_iter_fixed : prm->nitmax;
    HT3D_REQUIRE(prm->nitout >= 1, "nitout must be >= 1");
    for (int iter = 1; iter <= nmax; ++iter) {
        const bool chk = is_check(iter, prm->nitout);
        const bool storef = !chk && (iter == nmax || is_check(iter + 1, prm->nitout));
        sc.h1 = S.h1;
        sc.h2 = S.h2;
        sc.dtau = S.dtau;
        if (chk)
            launch_iter<double, MODE_CHECK>(ctx, L, cur, nxt, R, kx, ky, kz, PC, F0, F, sc, bc, nx, ny, nz, parts);
        else if (storef)
            launch_iter<double, MODE_STOREF>(ctx, L, cur, nxt, R, kx, ky, kz, PC, F0, F, sc, bc, nx, ny, nz, parts);
        else
            launch_iter<double, MODE_PLAIN>(ctx, L, cur, nxt, R, kx, ky, kz, PC, F0, F, sc, bc, nx, ny, nz, parts);
        std::swap(cur, nxt);
        it_done = iter;
        if (chk) {
            tree_sum3(ctx, parts, n, parts + 3 * n);
            if (C.update(S, prm, ctx->h_result[0], ctx->h_result[1], ctx->h_result[2], (double)n, iter,
                         n_iter_fixed <= 0))
                break;
        }
    }
    if (cur != X) {
        dim3 b(32, 8, 1), g((nx + 2 + 31) / 32, (ny + 2 + 7) / 8, nz + 2);
        HT3D_LAUNCH(ctx, k_copy_ex_faces<double>, g, b, 0, X, cur, nx, ny, nz);
    }
    C.fill(st, S, it_done);
    return C.status;
}



int ht3d_dyrel_solve_mixed(ht3d_ctx* ctx, double* X, const double* R, const double* kx, const double* ky,
                           const double* kz, double cX, double dx, double dy, double dz, const int* bc_type6,
                           const double* bc_val6, const ht3d_dyrel_params* prm, int n_iter_fixed, double* F,
                           double* F0, ht3d_dyrel_stats* st, int nx, int ny, int nz);

extern "C" int ht3d_dyrel_solve_dimless(ht3d_ctx* ctx, double* X_ex, const double* R, const double* kx,
                                        const double* ky, const double* kz, double cX, double dx, double dy, double dz,
                                        const int* bc_type6, const double* bc_val6, const ht3d_dyrel_params* prm,
                                        int n_iter_fixed, double* F, double* F0, int precision, ht3d_dyrel_stats* stats,
                                        int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        ht3d_check_dims(nx, ny, nz, 1);
        HT3D_REQUIRE(X_ex && R && kx && ky && kz && bc_type6 && bc_val6 && prm && F && F0, "null argument");
        HT3D_REQUIRE(prm->nitout >= 1 && prm->nitmax >= 1, "nitout and nitmax must be >= 1");
        if (precision == HT3D_FP64)
            return ht3d_dyrel_solve_fp64(ctx, X_ex, R, kx, ky, kz, cX, dx, dy, dz, bc_type6, bc_val6, prm, n_iter_fixed,
                                         F, F0, stats, nx, ny, nz);
        if (precision == HT3D_MIXED)
            return ht3d_dyrel_solve_mixed(ctx, X_ex, R, kx, ky, kz, cX, dx, dy, dz, bc_type6, bc_val6, prm,
                                          n_iter_fixed, F, F0, stats, nx, ny, nz);
        throw ht3d_error(HT3D_ERR_ARG, "unknown precision");
    });
}


extern "C" int ht3d_dyrel_iterate(ht3d_ctx* ctx, double* X_ex, const double* R, const double* kx, const double* ky,
                                  const double* kz, const double* PC, double* F0, double cX, double dx, double dy,
                                  double dz, const int* bc_type6, const double* bc_val6, double h1, double h2,
                                  double dtau, int n_iter, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        return dyrel_iterate_impl<double>(ctx, X_ex, R, kx, ky, kz, PC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1,
                                          h2, dtau, n_iter, nx, ny, nz, SLOT_AUX0);
    });
}


extern "C" int ht3d_dyrel_thermal_iterate(ht3d_ctx* ctx, int n_iter, double* T_ex, const double* Rt, const double* kx,
                                          const double* ky, const double* kz, const double* PC, double* F0,
                                          double _dt, double dx, double dy, double dz, const int* bc_type6,
                                          const double* bc_val6, double h1, double h2, double dtau, int nx, int ny,
                                          int nz) {
    return ht3d_dyrel_iterate(ctx, T_ex, Rt, kx, ky, kz, PC, F0, _dt, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau,
                              n_iter, nx, ny, nz);
}

extern "C" int ht3d_dyrel_darcy_iterate(ht3d_ctx* ctx, int n_iter, double* P_ex, const double* Rp, const double* kx,
                                        const double* ky, const double* kz, const double* PC, double* F0, double dx,
                                        double dy, double dz, const int* bc_type6, const double* bc_val6, double h1,
                                        double h2, double dtau, int nx, int ny, int nz) {
    return ht3d_dyrel_iterate(ctx, P_ex, Rp, kx, ky, kz, PC, F0, 0.0, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau,
                              n_iter, nx, ny, nz);
}
