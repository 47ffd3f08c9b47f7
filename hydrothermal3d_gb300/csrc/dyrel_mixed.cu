// Mixed-precision DYREL solver (FP32 inner iterations, FP64 defect correction).
#include "dyrel_common.cuh"

// ---------------------------------------------------------------------------
// Mixed-precision DYREL.
//
// The FP64 solution X (caller buffer) is only touched at check iterations.
// Between checks the iteration runs in FP32 on a correction field D with
// homogeneous boundary conditions:
//     F = (Rin + cX*D + div q(D)) * invPC,  F0 = h1 F0 + h2 F,  D -= dtau F0
// where Rin is the FP64 residual of X rounded to FP32.  At every check
// iteration of the reference schedule (iter % nitout == 0 || iter <= 2) one
// FP64 kernel folds D into X, recomputes the true FP64 residual
// (defect correction), evaluates the norms and Rayleigh-quotient sums in FP64,
// performs that iteration's update into D, and refreshes Rin.  The DYREL
// momentum F0 is stored in FP32 and carried across checks, so the iteration
// follows the FP64 one up to FP32 rounding within a check window while the
// stop test always sees the FP64 residual.
// ---------------------------------------------------------------------------
namespace {

__global__ void k_f64_to_f32(float* __restrict__ dst, const double* __restrict__ src, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = (float)src[t];
}
__global__ void k_f32_to_f64(double* __restrict__ dst, const float* __restrict__ src, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = (double)src[t];
}

// FP64 check iteration of the mixed solver (see above).
__global__ void __launch_bounds__(TX* TY) k_mixed_check(
    const double* __restrict__ Xin, double* __restrict__ Xout, const float* __restrict__ Din, float* __restrict__ Dout,
    const double* __restrict__ R, const double* __restrict__ kx, const double* __restrict__ ky,
    const double* __restrict__ kz, const double* __restrict__ invPC, float* __restrict__ F0,
    float* __restrict__ F32, double* __restrict__ F64, float* __restrict__ Rin, DyrelScal s, BC6<double> bc,
    int nx, int ny, int nz, int zchunk, double* __restrict__ partials) {
    const int i = blockIdx.x * TX + threadIdx.x;
    const int j = blockIdx.y * TY + threadIdx.y;
    const int k0 = blockIdx.z * zchunk;
    const int k1 = min(nz, k0 + zchunk);
    double acc[3] = {0.0, 0.0, 0.0};
    if (i < nx && j < ny && k0 < k1) {
        const int n1 = nx + 2, n2 = ny + 2;
        const long long pl = (long long)n1 * n2, cpl = (long long)nx * ny;
        const long long col = (i + 1) + (long long)n1 * (j + 1);
        const double* xcol = Xin + col;
        const float* dcol = Din + col;
        double* ocol = Xout + col;
        float* docol = Dout + col;
        const long long ccol = i + (long long)nx * j;
        const double* kxcol = kx + i + (long long)(nx + 1) * j;
        const double* kycol = ky + i + (long long)nx * j;
        const double* kzcol = kz + ccol;
        auto fold = [&](long long e) { return xcol[e] + (double)dcol[e]; };
        double xc = fold(pl * (k0 + 1));
        double xb = (k0 == 0) ? ghost(bc, 4, xc) : fold(pl * k0);
        double qB = -kzcol[cpl * k0] * (s._dz * (xc - xb));
        for (int k = k0; k < k1; ++k) {
            const long long e = pl * (k + 1);
            const double xf = (k == nz - 1) ? ghost(bc, 5, xc) : fold(e + pl);
            const double xw = (i == 0) ? ghost(bc, 0, xc) : fold(e - 1);
            const double xe = (i == nx - 1) ? ghost(bc, 1, xc) : fold(e + 1);
            const double xs = (j == 0) ? ghost(bc, 2, xc) : fold(e - n1);
            const double xn = (j == ny - 1) ? ghost(bc, 3, xc) : fold(e + n1);
            const long long c = ccol + cpl * k;
            const double qF = -kzcol[cpl * (k + 1)] * (s._dz * (xf - xc));
            const long long fxo = (long long)(nx + 1) * ny * k, fyo = (long long)nx * (ny + 1) * k;
            const double qW = -kxcol[fxo] * (s._dx * (xc - xw));
            const double qE = -kxcol[fxo + 1] * (s._dx * (xe - xc));
            const double qS = -kycol[fyo] * (s._dy * (xc - xs));
            const double qN = -kycol[fyo + nx] * (s._dy * (xn - xc));
            const double fu = R[c] + s.cX * xc + s._dx * (qE - qW) + s._dy * (qN - qS) + s._dz * (qF - qB);
            const double f = fu * invPC[c];
            const double f0 = s.h1 * (double)F0[c] + s.h2 * f;
            const double fit = (double)F32[c];
            const double d = s.dtau * f0;
            acc[0] += fabs(fu);
            acc[1] += -d * (f - fit);
            acc[2] += d * d;
            F0[c] = (float)f0;
            F32[c] = (float)f;
            F64[c] = f;
            Rin[c] = (float)fu;
            docol[e] = (float)(-d);
            ocol[e] = xc;
            if (i == 0) ocol[e - 1] = xw;
            if (i == nx - 1) ocol[e + 1] = xe;
            if (j == 0) ocol[e - n1] = xs;
            if (j == ny - 1) ocol[e + n1] = xn;
            if (k == 0) ocol[e - pl] = xb;
            if (k == nz - 1) ocol[e + pl] = xf;
            xb = xc;
            xc = xf;
            qB = qF;
        }
    }
    block_reduce<RED_SUM, 3>(acc);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const long long b = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
        partials[3 * b + 0] = acc[0];
        partials[3 * b + 1] = acc[1];
        partials[3 * b + 2] = acc[2];
    }
}

// X = X + D on inner cells, face ghosts = BC(folded inner)
__global__ void k_mixed_fold(double* __restrict__ X, const float* __restrict__ D, BC6<double> bc, int nx, int ny,
                             int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= nx || j >= ny || k >= nz) return;
    const int n1 = nx + 2, n2 = ny + 2;
    const long long pl = (long long)n1 * n2;
    const long long e = (i + 1) + (long long)n1 * (j + 1) + pl * (k + 1);
    const double x = X[e] + (double)D[e];
    X[e] = x;
    if (i == 0) X[e - 1] = ghost(bc, 0, x);
    if (i == nx - 1) X[e + 1] = ghost(bc, 1, x);
    if (j == 0) X[e - n1] = ghost(bc, 2, x);
    if (j == ny - 1) X[e + n1] = ghost(bc, 3, x);
    if (k == 0) X[e - pl] = ghost(bc, 4, x);
    if (k == nz - 1) X[e + pl] = ghost(bc, 5, x);
}

}  // namespace

int ht3d_dyrel_solve_mixed(ht3d_ctx* ctx, double* X, const double* R, const double* kx, const double* ky,
                           const double* kz, double cX, double dx, double dy, double dz, const int* bc_type6,
                           const double* bc_val6, const ht3d_dyrel_params* prm, int n_iter_fixed, double* F,
                           double* F0, ht3d_dyrel_stats* st, int nx, int ny, int nz) {
    const long long n = (long long)nx * ny * nz;
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    const long long nfx = (long long)(nx + 1) * ny * nz, nfy = (long long)nx * (ny + 1) * nz,
                    nfz = (long long)nx * ny * (nz + 1);
    double* invPC = (double*)ht3d_scratch(ctx, SLOT_PC, sizeof(double) * n);
    double* X2 = (double*)ht3d_scratch(ctx, SLOT_X2, sizeof(double) * nex);
    float* Da = (float*)ht3d_scratch(ctx, SLOT_F32_X, sizeof(float) * nex);
    float* Db = (float*)ht3d_scratch(ctx, SLOT_F32_X2, sizeof(float) * nex);
    float* F0s = (float*)ht3d_scratch(ctx, SLOT_F32_F0, sizeof(float) * n);
    float* Fs = (float*)ht3d_scratch(ctx, SLOT_F32_F, sizeof(float) * n);
    float* Rin = (float*)ht3d_scratch(ctx, SLOT_F32_R, sizeof(float) * n);
    float* iPC = (float*)ht3d_scratch(ctx, SLOT_F32_PC, sizeof(float) * n);
    float* kx32 = (float*)ht3d_scratch(ctx, SLOT_F32_KX, sizeof(float) * nfx);
    float* ky32 = (float*)ht3d_scratch(ctx, SLOT_F32_KY, sizeof(float) * nfy);
    float* kz32 = (float*)ht3d_scratch(ctx, SLOT_F32_KZ, sizeof(float) * nfz);
    IterLaunch L = iter_launch(ctx, nx, ny, nz, 0, 4);
    IterLaunch LC = iter_launch(ctx, nx, ny, nz, HT3D_DYREL_ZMARCH);  // layout of the FP64 check kernel
    const long long nparts = std::max<long long>(std::max(L.nblocks, LC.nblocks),
                                                 (long long)((nx + 31) / 32) * ((ny + 7) / 8) * nz);
    double* parts = (double*)ht3d_scratch(ctx, SLOT_PARTIALS, sizeof(double) * 3 * nparts);
    double* dres = (double*)ht3d_scratch(ctx, SLOT_RESULT, sizeof(double) * 64);

    BC6<double> bc;
    BC6<float> bch;  // homogeneous (correction) BCs
    for (int f = 0; f < 6; ++f) {
        HT3D_REQUIRE(bc_type6[f] == HT3D_BC_NEUMANN || bc_type6[f] == HT3D_BC_DIRICHLET, "face BC type must be 0 or 1");
        bc.dir[f] = bch.dir[f] = bc_type6[f];
        bc.val2[f] = 2.0 * bc_val6[f];
        bch.val2[f] = 0.0f;
    }
    {
        dim3 b(32, 8, 1), g((nx + 31) / 32, (ny + 7) / 8, nz);
        const double transient = cX != 0.0 ? 1.0 : 0.0, dt = cX != 0.0 ? 1.0 / cX : 1.0;
        HT3D_LAUNCH(ctx, k_dyrel_setup<1>, g, b, 0, kx, ky, kz, 1.0, transient, dt, dx, dy, dz, nx, ny, nz, invPC, parts);
        HT3D_LAUNCH(ctx, (k_reduce_partials<RED_MAX, 1>), 1, 1024, 0, parts, (int)(g.x * g.y * g.z), dres);
    }
    const unsigned gb = (unsigned)std::max(1, ctx->num_sms * 8);
    HT3D_LAUNCH(ctx, k_f64_to_f32, gb, 256, 0, iPC, invPC, n);
    HT3D_LAUNCH(ctx, k_f64_to_f32, gb, 256, 0, kx32, kx, nfx);
    HT3D_LAUNCH(ctx, k_f64_to_f32, gb, 256, 0, ky32, ky, nfy);
    HT3D_LAUNCH(ctx, k_f64_to_f32, gb, 256, 0, kz32, kz, nfz);
    HT3D_CUDA(cudaMemsetAsync(F0s, 0, sizeof(float) * n, ctx->stream));
    HT3D_CUDA(cudaMemsetAsync(Fs, 0, sizeof(float) * n, ctx->stream));
    HT3D_CUDA(cudaMemsetAsync(Da, 0, sizeof(float) * nex, ctx->stream));
    HT3D_CUDA(cudaMemsetAsync(Db, 0, sizeof(float) * nex, ctx->stream));
    ht3d_fetch_results(ctx, dres, 1);
    DyrelState S;
    dyrel_init_params(prm, ctx->h_result[0], S);

    DyrelScal sc;
    sc.cX = cX;
    sc._dx = 1.0 / dx;
    sc._dy = 1.0 / dy;
    sc._dz = 1.0 / dz;
    double* xcur = X;
    double* xnxt = X2;
    float* dcur = Da;
    float* dnxt = Db;
    double nF_abs = 0., nF_rel = 0., nF_ini = 0.;
    int it_done = 0, converged = 0, status = HT3D_OK, checks = 0;
    bool last_check = false;
    const int nmax = n_iter_fixed > 0 ? n_iter_fixed : prm->nitmax;
    const int refresh_every = ctx->mixed_refresh;
    for (int iter = 1; iter <= nmax; ++iter) {
        const bool chk = is_check(iter, prm->nitout);
        // defect-correction refresh between the reference's checks: fold D into X
        // and recompute the FP64 residual so the FP32 iteration never works
        // below its own precision (no stop test, no parameter update)
        const bool refresh = !chk && refresh_every > 0 && iter % refresh_every == 0;
        const bool storef = !chk && (iter == nmax || is_check(iter + 1, prm->nitout));
        sc.h1 = S.h1;
        sc.h2 = S.h2;
        sc.dtau = S.dtau;
        if (chk || refresh) {
            HT3D_LAUNCH(ctx, k_mixed_check, LC.grid, LC.block, 0, xcur, xnxt, dcur, dnxt, R, kx, ky, kz, invPC, F0s, Fs,
                        F, Rin, sc, bc, nx, ny, nz, LC.zchunk, parts);
            std::swap(xcur, xnxt);
        } else if (storef) {
            launch_iter<float, MODE_STOREF>(ctx, L, dcur, dnxt, Rin, kx32, ky32, kz32, iPC, F0s, Fs, sc, bch, nx, ny, nz, parts);
        } else {
            launch_iter<float, MODE_PLAIN>(ctx, L, dcur, dnxt, Rin, kx32, ky32, kz32, iPC, F0s, Fs, sc, bch, nx, ny, nz, parts);
        }
        std::swap(dcur, dnxt);
        it_done = iter;
        last_check = chk;
        if (chk) {
            ++checks;
            HT3D_LAUNCH(ctx, (k_reduce_partials<RED_SUM, 3>), 1, 1024, 0, parts, (int)LC.nblocks, dres);
            ht3d_fetch_results(ctx, dres, 3);
            const double s_abs = ctx->h_result[0], s_num = ctx->h_result[1], s_den = ctx->h_result[2];
            nF_abs = s_abs / (double)n / sqrt((double)n) * prm->norm_scale;
            if (iter == 1) nF_ini = nF_abs;
            nF_rel = nF_abs / nF_ini;
            if (std::isnan(nF_abs)) { status = HT3D_ERR_NAN; break; }
            if (nF_rel > 100) { status = HT3D_ERR_DIVERGED; break; }
            if (iter > 1) {
                S.lmin = fabs(s_num) / fabs(s_den);
                S.c = 2.0 * sqrt(S.lmin) * prm->cfact;
                S.h1 = (2 - S.c * S.dtau) / (2 + S.c * S.dtau);
                S.h2 = 2 * S.dtau / (2 + S.c * S.dtau);
            }
            if (n_iter_fixed <= 0 && (nF_abs < prm->tol_abs || nF_rel < prm->tol_rel)) { converged = 1; break; }
        }
    }
    // final fold of the correction into the FP64 solution
    {
        dim3 b(32, 8, 1), g((nx + 31) / 32, (ny + 7) / 8, nz);
        HT3D_LAUNCH(ctx, k_mixed_fold, g, b, 0, xcur, dcur, bc, nx, ny, nz);
    }
    if (xcur != X) {
        dim3 b(32, 8, 1), g((nx + 2 + 31) / 32, (ny + 2 + 7) / 8, nz + 2);
        HT3D_LAUNCH(ctx, k_copy_ex_faces<double>, g, b, 0, X, xcur, nx, ny, nz);
    }
    HT3D_LAUNCH(ctx, k_f32_to_f64, gb, 256, 0, F0, F0s, n);
    if (!last_check) HT3D_LAUNCH(ctx, k_f32_to_f64, gb, 256, 0, F, Fs, n);
    if (st) {
        st->iters = it_done; st->converged = converged; st->status = status; st->checks = checks;
        st->nF_abs = nF_abs; st->nF_rel = nF_rel; st->nF_ini = nF_ini; st->lambda_min = S.lmin;
        st->lambda_max = S.lmax; st->h1 = S.h1; st->h2 = S.h2; st->dtau = S.dtau;
    }
    return status;
}


extern "C" int ht3d_dyrel_iterate_f32(ht3d_ctx* ctx, float* X_ex, const float* R, const float* kx, const float* ky,
                                      const float* kz, const float* invPC, float* F0, double cX, double dx, double dy,
                                      double dz, const int* bc_type6, const double* bc_val6, double h1, double h2,
                                      double dtau, int n_iter, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        return dyrel_iterate_impl<float>(ctx, X_ex, R, kx, ky, kz, invPC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2,
                                         dtau, n_iter, nx, ny, nz, SLOT_AUX1);
    });
}
