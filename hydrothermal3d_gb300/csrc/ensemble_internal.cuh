// Internal interface between the ensemble time-step driver (ensemble.cu) and
// the batched mixed-precision DYREL solve (dyrel_mixed.cu).
#pragma once
#include "ht3d_internal.cuh"

// One instance of a batched solve: the arguments of ht3d_dyrel_solve_mixed.
struct EnsSolveInst {
    double* X;
    const double* R;
    const double* kx;
    const double* ky;
    const double* kz;
    double cX, dx, dy, dz;
    const int* bc_type6;
    const double* bc_val6;
    const ht3d_dyrel_params* prm;
    double* F;
    double* F0;
    ht3d_dyrel_stats* st;
    int nx, ny, nz;
    int status;  // in: nonzero = leave this instance alone; out: its solve status
};

// Solves every instance with status == 0 to its own stop test, all of them
// in lockstep: one launch per pseudo-iteration covers every instance still
// iterating.  Each instance's result is bit-identical to
// ht3d_dyrel_solve_mixed on the same context.  The instances must share
// nitout and nitmax.
void ht3d_ensemble_solve_mixed(ht3d_ctx* ctx, EnsSolveInst* inst, int n_inst);

// The body of ht3d_step_hrl (no status guard, no synchronisation).
int ht3d_step_hrl_impl(ht3d_ctx* ctx, double* Tc_ex, double* Pc_ex, const double* ktv, const double* kfv, double* Vx,
                       double* Vy, double* Vz, ht3d_hrl_params* p, ht3d_dyrel_stats* st_thermal,
                       ht3d_dyrel_stats* st_darcy, int precision, int nx, int ny, int nz);
void ht3d_weno5_advect_impl(ht3d_ctx* ctx, double* Tc_ex, const double* Vx, const double* Vy, const double* Vz,
                            double dt, double _dx, double _dy, double _dz, const int* bc_type6, const double* bc_val6,
                            int variant, int precision, int nx, int ny, int nz);
