// Ensemble of independent dimensionless HRL runs, one time step per call.
//
// The members' thermal solves iterate in lockstep through the batched mixed
// solve (one launch per pseudo-iteration over every member still iterating),
// then their Darcy solves; the per-member kernels around the solves are those
// of ht3d_step_hrl (step_kernels.cuh, compiled here with the same flags), so
// a member's result is bit-identical to a ht3d_step_hrl call on it.
#include "ensemble_internal.cuh"
#include "step_kernels.cuh"

namespace {

struct MemberBufs {
    double *R, *F, *F0, *Ty, *kx, *ky, *kz;
};

template <typename T>
T* carve(char* base, size_t& off, size_t count) {
    off = (off + 255) & ~(size_t)255;
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += sizeof(T) * (count ? count : 1);
    return p;
}

}  // namespace

extern "C" int ht3d_ensemble_step(ht3d_ctx* ctx, ht3d_instance* m, int n, int precision) {
    return ht3d_guard(ctx, [&]() {
        NvtxRange range("ht3d ensemble_step");
        HT3D_REQUIRE(m && n > 0, "no members");
        HT3D_REQUIRE(precision == HT3D_FP64 || precision == HT3D_MIXED, "unknown precision");
        for (int q = 0; q < n; ++q) {
            const ht3d_instance& I = m[q];
            ht3d_check_dims(I.nx, I.ny, I.nz, 1);
            HT3D_REQUIRE(I.Tc_ex && I.Pc_ex && I.ktv && I.kfv && I.Vx && I.Vy && I.Vz && I.params, "null argument");
            HT3D_REQUIRE(I.params->dt > 0.0, "dt must be positive");
        }
        int first = HT3D_OK;
        if (precision == HT3D_FP64) {
            for (int q = 0; q < n; ++q) {
                ht3d_instance& I = m[q];
                I.status = ht3d_step_hrl_impl(ctx, I.Tc_ex, I.Pc_ex, I.ktv, I.kfv, I.Vx, I.Vy, I.Vz, I.params,
                                              I.st_thermal, I.st_darcy, HT3D_FP64, I.nx, I.ny, I.nz);
                if (I.status && !first) first = I.status;
            }
            return first;
        }
        // per-member residual, flux and conductivity fields
        std::vector<MemberBufs> B(n);
        auto carve_all = [&](char* base) {
            size_t off = 0;
            for (int q = 0; q < n; ++q) {
                const long long nx = m[q].nx, ny = m[q].ny, nz = m[q].nz, nc = nx * ny * nz;
                B[q].R = carve<double>(base, off, nc);
                B[q].F = carve<double>(base, off, nc);
                B[q].F0 = carve<double>(base, off, nc);
                B[q].Ty = carve<double>(base, off, nx * (ny + 1) * nz);
                B[q].kx = carve<double>(base, off, (nx + 1) * ny * nz);
                B[q].ky = carve<double>(base, off, nx * (ny + 1) * nz);
                B[q].kz = carve<double>(base, off, nx * ny * (nz + 1));
            }
            return off;
        };
        carve_all((char*)ht3d_scratch(ctx, SLOT_ENS_STEP, carve_all(nullptr)));
        std::vector<EnsSolveInst> S(n);
        // thermal
        for (int q = 0; q < n; ++q) {
            ht3d_instance& I = m[q];
            const ht3d_hrl_params* p = I.params;
            const double _dt = 1.0 / p->dt;
            const dim3 gv = grid3(I.nx + 1, I.ny + 1, I.nz + 1, kBlock3);
            HT3D_LAUNCH(ctx, k_step_init_thermal, gv, kBlock3, 0, B[q].R, B[q].kx, B[q].ky, B[q].kz, I.Tc_ex, I.ktv, _dt,
                        I.nx, I.ny, I.nz);
            S[q] = EnsSolveInst{I.Tc_ex, B[q].R, B[q].kx, B[q].ky, B[q].kz, _dt, p->dx, p->dy, p->dz, p->thermal_bc,
                                p->thermal_val, &p->thermal, B[q].F, B[q].F0, I.st_thermal, I.nx, I.ny, I.nz, HT3D_OK};
        }
        ht3d_ensemble_solve_mixed(ctx, S.data(), n);
        for (int q = 0; q < n; ++q) m[q].status = S[q].status;
        // Darcy
        for (int q = 0; q < n; ++q) {
            ht3d_instance& I = m[q];
            const ht3d_hrl_params* p = I.params;
            S[q].status = I.status;
            if (I.status) continue;
            const dim3 gv = grid3(I.nx + 1, I.ny + 1, I.nz + 1, kBlock3), gc = grid3(I.nx, I.ny, I.nz, kBlock3);
            HT3D_LAUNCH(ctx, k_step_init_darcy, gv, kBlock3, 0, B[q].Ty, B[q].kx, B[q].ky, B[q].kz, I.Tc_ex, I.kfv,
                        p->kill_ns, I.nx, I.ny, I.nz);
            HT3D_LAUNCH(ctx, k_step_rp, gc, kBlock3, 0, B[q].R, B[q].ky, B[q].Ty, p->Ra, 1.0 / p->dy, I.nx, I.ny, I.nz);
            S[q] = EnsSolveInst{I.Pc_ex, B[q].R, B[q].kx, B[q].ky, B[q].kz, 0.0, p->dx, p->dy, p->dz, p->darcy_bc,
                                p->darcy_val, &p->darcy, B[q].F, B[q].F0, I.st_darcy, I.nx, I.ny, I.nz, HT3D_OK};
        }
        ht3d_ensemble_solve_mixed(ctx, S.data(), n);
        for (int q = 0; q < n; ++q) m[q].status = S[q].status;
        // velocity, advection and the members' max |V| for the adaptive dt
        double* vres = (double*)ht3d_scratch(ctx, SLOT_RESULT, sizeof(double) * 64);
        std::vector<double> vmax(3 * (size_t)n, 0.0);
        int pending = 0;
        auto flush = [&](int upto) {
            if (!pending) return;
            HT3D_CUDA(cudaMemcpyAsync(ctx->h_result, vres, sizeof(double) * 3 * pending, cudaMemcpyDeviceToHost,
                                      ctx->stream));
            HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
            for (int r = 0; r < pending; ++r)
                for (int c = 0; c < 3; ++c) vmax[3 * (size_t)(upto - pending + r) + c] = ctx->h_result[3 * r + c];
            pending = 0;
        };
        std::vector<int> order;
        for (int q = 0; q < n; ++q) {
            ht3d_instance& I = m[q];
            if (I.status) continue;
            const ht3d_hrl_params* p = I.params;
            const double _dx = 1.0 / p->dx, _dy = 1.0 / p->dy, _dz = 1.0 / p->dz;
            const dim3 gv = grid3(I.nx + 1, I.ny + 1, I.nz + 1, kBlock3);
            HT3D_LAUNCH(ctx, k_step_vel, gv, kBlock3, 0, I.Vx, I.Vy, I.Vz, B[q].kx, B[q].ky, B[q].kz, I.Pc_ex, B[q].Ty,
                        p->Ra, _dx, _dy, _dz, I.nx, I.ny, I.nz);
            if (p->advection)
                ht3d_weno5_advect_impl(ctx, I.Tc_ex, I.Vx, I.Vy, I.Vz, p->dt, _dx, _dy, _dz, p->weno_bc, p->weno_val,
                                       p->weno_variant, HT3D_MIXED, I.nx, I.ny, I.nz);
            if (p->dt_adapt) order.push_back(q);
        }
        // max |V| of up to 21 members per fetch (64 result slots)
        for (size_t r = 0; r < order.size(); ++r) {
            const ht3d_instance& I = m[order[r]];
            const long long nx = I.nx, ny = I.ny, nz = I.nz;
            ht3d_reduce_device(ctx, I.Vx, (nx + 1) * ny * nz, RED_MAX_ABS, vres + 3 * pending);
            ht3d_reduce_device(ctx, I.Vy, nx * (ny + 1) * nz, RED_MAX_ABS, vres + 3 * pending + 1);
            ht3d_reduce_device(ctx, I.Vz, nx * ny * (nz + 1), RED_MAX_ABS, vres + 3 * pending + 2);
            if (++pending == 21) flush((int)r + 1);
        }
        flush((int)order.size());
        for (size_t r = 0; r < order.size(); ++r) {
            ht3d_hrl_params* p = m[order[r]].params;
            const double v = std::max(std::max(vmax[3 * r], vmax[3 * r + 1]), vmax[3 * r + 2]);
            p->dt = p->dt_fact * 1.0 / 6.1 * std::min(std::min(p->dx, p->dy), p->dz) / v;
            if (p->dt_max > 0.0 && p->dt > p->dt_max) p->dt = p->dt_max;
        }
        for (int q = 0; q < n; ++q)
            if (m[q].status && !first) first = m[q].status;
        return first;
    });
}
