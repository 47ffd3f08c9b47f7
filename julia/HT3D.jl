# Generated by julia/generate.py from include/ht3d.h: do not edit.
#
# Julia binding of libht3d.so, the GB300 implementation of HydroThermal3D's
# pseudo-transient kernels.  A driver replaces `@parallel Kernel!(args...)` by
# `HT3D.Kernel!(args...)` with the same arguments (CuArray{Float64,3} in the
# reference's staggering); grid sizes are inferred from the array shapes, a
# wrong shape throws ArgumentError, a non-zero status Ht3dError.  Every call
# runs on the stream of its Context (by default one created on CUDA.jl's task
# stream) and returns after the kernel finished, like @parallel.
module HT3D

using CUDA

const libht3d = get(ENV, "HT3D_LIB", joinpath(@__DIR__, "..", "hydrothermal3d_gb300", "libht3d.so"))
const CU_NULL = CuPtr{Cdouble}(0)

# ---------------------------------------------------------------- constants
const ABI_VERSION = Cint(1)
const OK = Cint(0)
const ERR_ARG = Cint(1)
const ERR_CUDA = Cint(2)
const ERR_NAN = Cint(3)
const ERR_DIVERGED = Cint(4)
const ERR_MAXITER = Cint(5)
const ERR_TIMEOUT = Cint(6)
const ERR_NOMEM = Cint(7)
const ERR_SCRATCH = Cint(8)
const ERR_IO = Cint(9)
const FP64 = Cint(0)
const MIXED = Cint(1)
const BC_NEUMANN = Cint(0)
const BC_DIRICHLET = Cint(1)
const BC_PERIODIC = Cint(2)
const WENO_V1 = Cint(0)
const WENO_V2_REF = Cint(1)
const WENO_V2_FIXED = Cint(2)
const TUNE_DYREL_VARIANT = Cint(1)
const DYREL_AUTO = Cint(0)
const DYREL_ZMARCH = Cint(1)
const DYREL_CELL = Cint(2)
const TUNE_MIXED_REFRESH = Cint(2)
const TUNE_TIME_INNER = Cint(3)
const TUNE_ENS_BLOCK = Cint(4)
const TUNE_ENS_GRAPH = Cint(5)
const TUNE_TEMPORAL = Cint(6)
const TUNE_ENS_TILE = Cint(8)
const TUNE_WAIT_TEST = Cint(7)

# ---------------------------------------------------------------- structs
# ht3d_dyrel_params (include/ht3d.h)
Base.@kwdef struct DyrelParams
    tol_abs::Cdouble = 0.0
    tol_rel::Cdouble = 0.0
    nitmax::Cint = Cint(0)
    nitout::Cint = Cint(0)
    cfl::Cdouble = 0.0
    cfact::Cdouble = 0.0
    lmin_ratio::Cdouble = 0.0
    norm_scale::Cdouble = 0.0
end

# ht3d_dyrel_stats (include/ht3d.h)
Base.@kwdef struct DyrelStats
    iters::Cint = Cint(0)
    converged::Cint = Cint(0)
    status::Cint = Cint(0)
    checks::Cint = Cint(0)
    nF_abs::Cdouble = 0.0
    nF_rel::Cdouble = 0.0
    nF_ini::Cdouble = 0.0
    lambda_min::Cdouble = 0.0
    lambda_max::Cdouble = 0.0
    h1::Cdouble = 0.0
    h2::Cdouble = 0.0
    dtau::Cdouble = 0.0
end

# ht3d_hrl_params (include/ht3d.h)
Base.@kwdef struct HrlParams
    Ra::Cdouble = 0.0
    dx::Cdouble = 0.0
    dy::Cdouble = 0.0
    dz::Cdouble = 0.0
    dt::Cdouble = 0.0
    Tbot::Cdouble = 0.0
    Ttop::Cdouble = 0.0
    thermal_bc::NTuple{6, Cint} = ntuple(_ -> Cint(0), 6)
    thermal_val::NTuple{6, Cdouble} = ntuple(_ -> 0.0, 6)
    darcy_bc::NTuple{6, Cint} = ntuple(_ -> Cint(0), 6)
    darcy_val::NTuple{6, Cdouble} = ntuple(_ -> 0.0, 6)
    weno_bc::NTuple{6, Cint} = ntuple(_ -> Cint(0), 6)
    weno_val::NTuple{6, Cdouble} = ntuple(_ -> 0.0, 6)
    weno_variant::Cint = Cint(0)
    kill_ns::Cint = Cint(0)
    dt_adapt::Cint = Cint(0)
    advection::Cint = Cint(0)
    dt_fact::Cdouble = 0.0
    thermal::DyrelParams = DyrelParams()
    darcy::DyrelParams = DyrelParams()
    dt_max::Cdouble = 0.0
end

# ht3d_v18_params (include/ht3d.h)
Base.@kwdef struct V18Params
    dx::Cdouble = 0.0
    dy::Cdouble = 0.0
    dz::Cdouble = 0.0
    ymin::Cdouble = 0.0
    dt::Cdouble = 0.0
    time::Cdouble = 0.0
    phi_i::Cdouble = 0.0
    k_fact::Cdouble = 0.0
    delta::Cdouble = 0.0
    g::Cdouble = 0.0
    Qt::Cdouble = 0.0
    qyS::Cdouble = 0.0
    Ttop::Cdouble = 0.0
    Tbot::Cdouble = 0.0
    Ptop::Cdouble = 0.0
    Pbot::Cdouble = 0.0
    T_pluton::Cdouble = 0.0
    C_adv::Cdouble = 0.0
    sc_T::Cdouble = 0.0
    sc_L::Cdouble = 0.0
    sc_t::Cdouble = 0.0
    sc_eta::Cdouble = 0.0
    sc_sigma::Cdouble = 0.0
    sc_rho::Cdouble = 0.0
    sc_C::Cdouble = 0.0
    sc_kt::Cdouble = 0.0
    it::Cint = Cint(0)
    thermal::Cint = Cint(0)
    hydro::Cint = Cint(0)
    advection::Cint = Cint(0)
    dt_constant::Cint = Cint(0)
    weno_variant::Cint = Cint(0)
    thermal_dyrel::DyrelParams = DyrelParams()
    darcy_dyrel::DyrelParams = DyrelParams()
    n_adv::Cint = Cint(0)
    pad_::Cint = Cint(0)
end

# ht3d_khaled_geom (include/ht3d.h)
Base.@kwdef struct KhaledGeom
    y_plateau::Cdouble = 0.0
    surf_a1::Cdouble = 0.0
    surf_b1::Cdouble = 0.0
    fault::NTuple{4, NTuple{6, Cdouble}} = ntuple(_ -> ntuple(_ -> 0.0, 6), 4)
end

# ht3d_post_params (include/ht3d.h)
Base.@kwdef struct PostParams
    phi0::Cdouble = 0.0
    scale_T::Cdouble = 0.0
    scale_sigma::Cdouble = 0.0
    scale_V::Cdouble = 0.0
    scale_L::Cdouble = 0.0
    k_fact::Cdouble = 0.0
    ymin::Cdouble = 0.0
    dy::Cdouble = 0.0
    delta::Cdouble = 0.0
end

# ht3d_post_fields (include/ht3d.h)
Base.@kwdef struct PostFields
    phase::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    pressure::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    temperature::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    vx::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    vy::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    vz::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    k_thermal::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    heat_capacity::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    permeability::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    density::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    viscosity::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    peclet::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
end

# ht3d_instance (include/ht3d.h)
Base.@kwdef struct Instance
    Tc_ex::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    Pc_ex::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    ktv::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    kfv::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    Vx::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    Vy::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    Vz::CuPtr{Cdouble} = CuPtr{Cdouble}(0)
    params::Ptr{HrlParams} = Ptr{HrlParams}(C_NULL)
    st_thermal::Ptr{DyrelStats} = Ptr{DyrelStats}(C_NULL)
    st_darcy::Ptr{DyrelStats} = Ptr{DyrelStats}(C_NULL)
    nx::Cint = Cint(0)
    ny::Cint = Cint(0)
    nz::Cint = Cint(0)
    status::Cint = Cint(0)
end

# ---------------------------------------------------------------- C entry points (one per prototype)
module C
using CUDA
import ..HT3D: libht3d, DyrelParams, DyrelStats, HrlParams, V18Params, KhaledGeom, PostParams, PostFields, Instance

ht3d_abi_version() =
    ccall((:ht3d_abi_version, libht3d), Cint, ())
ht3d_status_string(status) =
    ccall((:ht3d_status_string, libht3d), Cstring, (Cint,), status)
ht3d_ctx_create(out, device, stream) =
    ccall((:ht3d_ctx_create, libht3d), Cint, (Ref{Ptr{Cvoid}}, Cint, Ptr{Cvoid}), out, device, stream)
ht3d_ctx_destroy(ctx) =
    ccall((:ht3d_ctx_destroy, libht3d), Cint, (Ptr{Cvoid},), ctx)
ht3d_ctx_set_stream(ctx, stream) =
    ccall((:ht3d_ctx_set_stream, libht3d), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx, stream)
ht3d_ctx_set_sync(ctx, sync_each_call) =
    ccall((:ht3d_ctx_set_sync, libht3d), Cint, (Ptr{Cvoid}, Cint), ctx, sync_each_call)
ht3d_ctx_synchronize(ctx) =
    ccall((:ht3d_ctx_synchronize, libht3d), Cint, (Ptr{Cvoid},), ctx)
ht3d_ctx_set_tuning(ctx, key, value) =
    ccall((:ht3d_ctx_set_tuning, libht3d), Cint, (Ptr{Cvoid}, Cint, Cint), ctx, key, value)
ht3d_ctx_launch_count(ctx) =
    ccall((:ht3d_ctx_launch_count, libht3d), Culonglong, (Ptr{Cvoid},), ctx)
ht3d_ctx_inner_timing(ctx, ms, launches, reset) =
    ccall((:ht3d_ctx_inner_timing, libht3d), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Culonglong}, Cint), ctx, ms, launches, reset)
ht3d_ctx_last_error(ctx) =
    ccall((:ht3d_ctx_last_error, libht3d), Cstring, (Ptr{Cvoid},), ctx)
ht3d_sizeof_dyrel_params() =
    ccall((:ht3d_sizeof_dyrel_params, libht3d), Cint, ())
ht3d_sizeof_dyrel_stats() =
    ccall((:ht3d_sizeof_dyrel_stats, libht3d), Cint, ())
ht3d_sizeof_hrl_params() =
    ccall((:ht3d_sizeof_hrl_params, libht3d), Cint, ())
ht3d_sizeof_instance() =
    ccall((:ht3d_sizeof_instance, libht3d), Cint, ())
ht3d_sizeof_v18_params() =
    ccall((:ht3d_sizeof_v18_params, libht3d), Cint, ())
ht3d_reduce(ctx, a, n, op, out) =
    ccall((:ht3d_reduce, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, Clonglong, Cint, Ptr{Cdouble}), ctx, a, n, op, out)
ht3d_Init_vel(ctx, Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty, Ra, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_Init_vel, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty, Ra, _dx, _dy, _dz, nx, ny, nz)
ht3d_InitDarcy(ctx, Ty, kx, ky, kz, Tc_ex, kfv, _dt, nx, ny, nz) =
    ccall((:ht3d_InitDarcy, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Cint), ctx, Ty, kx, ky, kz, Tc_ex, kfv, _dt, nx, ny, nz)
ht3d_Compute_Rp(ctx, Rp, ky, Ty, Ra, _dy, nx, ny, nz) =
    ccall((:ht3d_Compute_Rp, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint), ctx, Rp, ky, Ty, Ra, _dy, nx, ny, nz)
ht3d_InitThermal(ctx, Rt, kx, ky, kz, Tc_ex, ktv, _dt, nx, ny, nz) =
    ccall((:ht3d_InitThermal, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Cint), ctx, Rt, kx, ky, kz, Tc_ex, ktv, _dt, nx, ny, nz)
ht3d_ComputeFlux(ctx, qx, qy, qz, kx, ky, kz, A, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_ComputeFlux, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, qx, qy, qz, kx, ky, kz, A, _dx, _dy, _dz, nx, ny, nz)
ht3d_UpdateT(ctx, F, T, R, qx, qy, qz, _dt, dtau, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_UpdateT, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, F, T, R, qx, qy, qz, _dt, dtau, _dx, _dy, _dz, nx, ny, nz)
ht3d_ResidualDiffusion(ctx, F, R, qx, qy, qz, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_ResidualDiffusion, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, F, R, qx, qy, qz, _dx, _dy, _dz, nx, ny, nz)
ht3d_ResidualDiffusionTransient(ctx, F, T, R, qx, qy, qz, _dt, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_ResidualDiffusionTransient, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, F, T, R, qx, qy, qz, _dt, _dx, _dy, _dz, nx, ny, nz)
ht3d_UpdateP(ctx, F0, P, F, dampx, dtau, nx, ny, nz) =
    ccall((:ht3d_UpdateP, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint), ctx, F0, P, F, dampx, dtau, nx, ny, nz)
ht3d_DYRELUpdate(ctx, F0, X, F, h1, h2, dtau, nx, ny, nz) =
    ccall((:ht3d_DYRELUpdate, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, F0, X, F, h1, h2, dtau, nx, ny, nz)
ht3d_SetPressureBCs(ctx, Pc_ex, Pbot, Ptop, nx, ny, nz) =
    ccall((:ht3d_SetPressureBCs, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint), ctx, Pc_ex, Pbot, Ptop, nx, ny, nz)
ht3d_SetFaceBCs(ctx, X_ex, bc_type6, bc_val6, nx, ny, nz) =
    ccall((:ht3d_SetFaceBCs, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, Ptr{Cint}, Ptr{Cdouble}, Cint, Cint, Cint), ctx, X_ex, bc_type6, bc_val6, nx, ny, nz)
ht3d_KillNorthSouthFluxes(ctx, Ty, nx, ny, nz) =
    ccall((:ht3d_KillNorthSouthFluxes, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, Ty, nx, ny, nz)
ht3d_ResetA(ctx, A, B, n) =
    ccall((:ht3d_ResetA, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Clonglong), ctx, A, B, n)
ht3d_Cpy_inn_to_all(ctx, A, B_ex, nx, ny, nz) =
    ccall((:ht3d_Cpy_inn_to_all, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, A, B_ex, nx, ny, nz)
ht3d_Cpy_all_to_inn(ctx, A_ex, B, nx, ny, nz) =
    ccall((:ht3d_Cpy_all_to_inn, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, A_ex, B, nx, ny, nz)
ht3d_ArrayEqualArray(ctx, A, B, n) =
    ccall((:ht3d_ArrayEqualArray, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Clonglong), ctx, A, B, n)
ht3d_Multiply(ctx, a, b, c, n) =
    ccall((:ht3d_Multiply, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Clonglong), ctx, a, b, c, n)
ht3d_GershgorinPoisson(ctx, G, D, rhoC_eff, kx, ky, kz, transient, dt, dx, dy, dz, nx, ny, nz) =
    ccall((:ht3d_GershgorinPoisson, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, G, D, rhoC_eff, kx, ky, kz, transient, dt, dx, dy, dz, nx, ny, nz)
ht3d_GershgorinHydro(ctx, G, phidrhodP, kx, ky, kz, transient, dt, dx, dy, dz, nx, ny, nz) =
    ccall((:ht3d_GershgorinHydro, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, G, phidrhodP, kx, ky, kz, transient, dt, dx, dy, dz, nx, ny, nz)
ht3d_SwapDYREL(ctx, Xc, Yc, X0c_ex, Y0c, nx, ny, nz) =
    ccall((:ht3d_SwapDYREL, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, Xc, Yc, X0c_ex, Y0c, nx, ny, nz)
ht3d_RayleighQuotientNumerator(ctx, G, Fc0, Fcit, Fc, dtau, n) =
    ccall((:ht3d_RayleighQuotientNumerator, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Clonglong), ctx, G, Fc0, Fcit, Fc, dtau, n)
ht3d_RayleighQuotientDenominator(ctx, G, Fc0, dtau, n) =
    ccall((:ht3d_RayleighQuotientDenominator, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Clonglong), ctx, G, Fc0, dtau, n)
ht3d_ComputeThermalConductivity(ctx, ktv, Tce, phv, phi0, scale_kt, scale_T, nx, ny, nz) =
    ccall((:ht3d_ComputeThermalConductivity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, ktv, Tce, phv, phi0, scale_kt, scale_T, nx, ny, nz)
ht3d_ComputeHydroConductivity(ctx, kfv, Tce, Pce, phv, ymin, dy, k_fact, delta, scale_sigma, scale_T, scale_L, scale_t, scale_eta, mode, kmul_v, nx, ny, nz) =
    ccall((:ht3d_ComputeHydroConductivity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, kfv, Tce, Pce, phv, ymin, dy, k_fact, delta, scale_sigma, scale_T, scale_L, scale_t, scale_eta, mode, kmul_v, nx, ny, nz)
ht3d_ComputeFluidDensity(ctx, rhofv, Tce, Pce, phv, scale_sigma, scale_T, scale_rho, nx, ny, nz) =
    ccall((:ht3d_ComputeFluidDensity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, rhofv, Tce, Pce, phv, scale_sigma, scale_T, scale_rho, nx, ny, nz)
ht3d_SmoothConductivityV2C(ctx, ktc, ktv, nx, ny, nz) =
    ccall((:ht3d_SmoothConductivityV2C, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, ktc, ktv, nx, ny, nz)
ht3d_SmoothConductivityC2V(ctx, ktv, ktc, nx, ny, nz) =
    ccall((:ht3d_SmoothConductivityC2V, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, ktv, ktc, nx, ny, nz)
ht3d_InitConductivity(ctx, kx, ky, kz, ktv, nx, ny, nz) =
    ccall((:ht3d_InitConductivity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, kx, ky, kz, ktv, nx, ny, nz)
ht3d_ComputeRhoCeffective(ctx, rhoC_eff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho, nx, ny, nz) =
    ccall((:ht3d_ComputeRhoCeffective, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, rhoC_eff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho, nx, ny, nz)
ht3d_ResidualTemperatureLinearised(ctx, F, Tc_ex, Tc_old, rhoC_eff, phc_ex, PC, qx, qy, qz, Qt, transient, _dt, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_ResidualTemperatureLinearised, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, F, Tc_ex, Tc_old, rhoC_eff, phc_ex, PC, qx, qy, qz, Qt, transient, _dt, _dx, _dy, _dz, nx, ny, nz)
ht3d_SetTemperatureBCs(ctx, Tc_ex, ky, wN, phc_ex, qyS, _dy, kS, TS, TN, y_plateau, a2, b2, dTdy, dx, dy, sticky_air, sca_T, sca_kT, phi_i, nx, ny, nz) =
    ccall((:ht3d_SetTemperatureBCs, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, Tc_ex, ky, wN, phc_ex, qyS, _dy, kS, TS, TN, y_plateau, a2, b2, dTdy, dx, dy, sticky_air, sca_T, sca_kT, phi_i, nx, ny, nz)
ht3d_SetPressureBCs_dim(ctx, Pc_ex, wN, phc_ex, PS, PN, y_plateau, a2, b2, rhof, g, dx, dy, sticky_air, nx, ny, nz) =
    ccall((:ht3d_SetPressureBCs_dim, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint, Cint), ctx, Pc_ex, wN, phc_ex, PS, PN, y_plateau, a2, b2, rhof, g, dx, dy, sticky_air, nx, ny, nz)
ht3d_PhiRhof(ctx, phirhofc, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz) =
    ccall((:ht3d_PhiRhof, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, phirhofc, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz)
ht3d_PhiRhofOld(ctx, phirhofc, Tc0, Pc0, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz) =
    ccall((:ht3d_PhiRhofOld, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, phirhofc, Tc0, Pc0, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz)
ht3d_PhiDrhodP(ctx, phidrhodP, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz) =
    ccall((:ht3d_PhiDrhodP, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, phidrhodP, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz)
ht3d_ComputeDarcyFlux(ctx, qx, qy, qz, rhofv, kx, ky, kz, Pf, g, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_ComputeDarcyFlux, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, qx, qy, qz, rhofv, kx, ky, kz, Pf, g, _dx, _dy, _dz, nx, ny, nz)
ht3d_ResidualFluidPressure(ctx, F, phc_ex, phirhofc, phirhofc0, PC, qx, qy, qz, transient, _dt, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_ResidualFluidPressure, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, F, phc_ex, phirhofc, phirhofc0, PC, qx, qy, qz, transient, _dt, _dx, _dy, _dz, nx, ny, nz)
ht3d_Init_vel_dim(ctx, Vx, Vy, Vz, qx, qy, qz, rhofv, nx, ny, nz) =
    ccall((:ht3d_Init_vel_dim, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, Vx, Vy, Vz, qx, qy, qz, rhofv, nx, ny, nz)
ht3d_material_law(ctx, which, a, b, out, n) =
    ccall((:ht3d_material_law, libht3d), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Clonglong), ctx, which, a, b, out, n)
ht3d_VPlusMinus(ctx, Vm, Vp, V, axis, nx, ny, nz) =
    ccall((:ht3d_VPlusMinus, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint, Cint), ctx, Vm, Vp, V, axis, nx, ny, nz)
ht3d_dFdx_Weno5(ctx, dFdxi, V1, V2, V3, V4, V5, n) =
    ccall((:ht3d_dFdx_Weno5, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Clonglong), ctx, dFdxi, V1, V2, V3, V4, V5, n)
ht3d_Gradients_Weno5(ctx, v1, v2, v3, v4, v5, Fc_exxx, axis, sign, _dx, _dy, _dz, nx, ny, nz) =
    ccall((:ht3d_Gradients_Weno5, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, v1, v2, v3, v4, v5, Fc_exxx, axis, sign, _dx, _dy, _dz, nx, ny, nz)
ht3d_Boundaries_Weno5(ctx, Fc_exxx, Fc, axis, type_L, val_L, type_R, val_R, fc_ghosted, nx, ny, nz) =
    ccall((:ht3d_Boundaries_Weno5, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cdouble, Cint, Cdouble, Cint, Cint, Cint, Cint), ctx, Fc_exxx, Fc, axis, type_L, val_L, type_R, val_R, fc_ghosted, nx, ny, nz)
ht3d_Advect_v1(ctx, Fc, Vxp, dTdxm, Vxm, dTdxp, dt, n) =
    ccall((:ht3d_Advect_v1, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Clonglong), ctx, Fc, Vxp, dTdxm, Vxm, dTdxp, dt, n)
ht3d_TimeAveraging_v1(ctx, Fc, Fold, order, n) =
    ccall((:ht3d_TimeAveraging_v1, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Clonglong), ctx, Fc, Fold, order, n)
ht3d_Advect_v2(ctx, Fc_ex, X_exxx, V, axis, dt, _dx, _dy, _dz, quirk, nx, ny, nz) =
    ccall((:ht3d_Advect_v2, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint, Cint), ctx, Fc_ex, X_exxx, V, axis, dt, _dx, _dy, _dz, quirk, nx, ny, nz)
ht3d_TimeAveraging_v2(ctx, Fc_ex, Fold, order, nx, ny, nz) =
    ccall((:ht3d_TimeAveraging_v2, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Cint), ctx, Fc_ex, Fold, order, nx, ny, nz)
ht3d_weno5_advect(ctx, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant, precision, nx, ny, nz) =
    ccall((:ht3d_weno5_advect, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cint}, Ptr{Cdouble}, Cint, Cint, Cint, Cint, Cint), ctx, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant, precision, nx, ny, nz)
ht3d_weno5_advect_f32(ctx, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant, nx, ny, nz) =
    ccall((:ht3d_weno5_advect_f32, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cint}, Ptr{Cdouble}, Cint, Cint, Cint, Cint), ctx, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant, nx, ny, nz)
ht3d_dyrel_solve_dimless(ctx, X_ex, R, kx, ky, kz, cX, dx, dy, dz, bc_type6, bc_val6, prm, n_iter_fixed, F, F0, precision, stats, nx, ny, nz) =
    ccall((:ht3d_dyrel_solve_dimless, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cint}, Ptr{Cdouble}, Ref{DyrelParams}, Cint, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Ref{DyrelStats}, Cint, Cint, Cint), ctx, X_ex, R, kx, ky, kz, cX, dx, dy, dz, bc_type6, bc_val6, prm, n_iter_fixed, F, F0, precision, stats, nx, ny, nz)
ht3d_dyrel_iterate(ctx, X_ex, R, kx, ky, kz, PC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter, nx, ny, nz) =
    ccall((:ht3d_dyrel_iterate, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cint}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint, Cint), ctx, X_ex, R, kx, ky, kz, PC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter, nx, ny, nz)
ht3d_dyrel_thermal_iterate(ctx, n_iter, T_ex, Rt, kx, ky, kz, PC, F0, _dt, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, nx, ny, nz) =
    ccall((:ht3d_dyrel_thermal_iterate, libht3d), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cint}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, n_iter, T_ex, Rt, kx, ky, kz, PC, F0, _dt, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, nx, ny, nz)
ht3d_dyrel_darcy_iterate(ctx, n_iter, P_ex, Rp, kx, ky, kz, PC, F0, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, nx, ny, nz) =
    ccall((:ht3d_dyrel_darcy_iterate, libht3d), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Ptr{Cint}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, n_iter, P_ex, Rp, kx, ky, kz, PC, F0, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, nx, ny, nz)
ht3d_dyrel_iterate_f32(ctx, X_ex, R, kx, ky, kz, invPC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter, nx, ny, nz) =
    ccall((:ht3d_dyrel_iterate_f32, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cint}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint, Cint), ctx, X_ex, R, kx, ky, kz, invPC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter, nx, ny, nz)
ht3d_dyrel_iterate_noalloc(X_ex, R, kx, ky, kz, PC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter, nx, ny, nz, stream) =
    ccall((:ht3d_dyrel_iterate_noalloc, libht3d), Cint, (CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cint}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint, Cint, Ptr{Cvoid}), X_ex, R, kx, ky, kz, PC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter, nx, ny, nz, stream)
ht3d_step_hrl(ctx, Tc_ex, Pc_ex, ktv, kfv, Vx, Vy, Vz, p, st_thermal, st_darcy, precision, nx, ny, nz) =
    ccall((:ht3d_step_hrl, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ref{HrlParams}, Ref{DyrelStats}, Ref{DyrelStats}, Cint, Cint, Cint, Cint), ctx, Tc_ex, Pc_ex, ktv, kfv, Vx, Vy, Vz, p, st_thermal, st_darcy, precision, nx, ny, nz)
ht3d_ensemble_step(ctx, members, n_members, precision) =
    ccall((:ht3d_ensemble_step, libht3d), Cint, (Ptr{Cvoid}, Ptr{Instance}, Cint, Cint), ctx, members, n_members, precision)
ht3d_SetInitialConditions_Khaled(ctx, phc_ex, phv, wN, geom, Tc_ex, Pc_ex, Tbot, Ttop, Pbot, Ptop, xmin, ymin, zmin, xmax, ymax, zmax, L, nx, ny, nz) =
    ccall((:ht3d_SetInitialConditions_Khaled, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ref{KhaledGeom}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, phc_ex, phv, wN, geom, Tc_ex, Pc_ex, Tbot, Ttop, Pbot, Ptop, xmin, ymin, zmin, xmax, ymax, zmax, L, nx, ny, nz)
ht3d_step_v18(ctx, Tc_ex, Pc_ex, phc_ex, phv, wN, kmul_v, Vx, Vy, Vz, p, st_thermal, st_darcy, nx, ny, nz) =
    ccall((:ht3d_step_v18, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ref{V18Params}, Ref{DyrelStats}, Ref{DyrelStats}, Cint, Cint, Cint), ctx, Tc_ex, Pc_ex, phc_ex, phv, wN, kmul_v, Vx, Vy, Vz, p, st_thermal, st_darcy, nx, ny, nz)
ht3d_Phase(ctx, X, phc_ex, nx, ny, nz) =
    ccall((:ht3d_Phase, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, X, phc_ex, nx, ny, nz)
ht3d_Pressure(ctx, X, Pc_ex, phc_ex, scale_sigma, nx, ny, nz) =
    ccall((:ht3d_Pressure, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Cint), ctx, X, Pc_ex, phc_ex, scale_sigma, nx, ny, nz)
ht3d_Temperature(ctx, X, Tc_ex, phc_ex, scale_T, nx, ny, nz) =
    ccall((:ht3d_Temperature, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Cint), ctx, X, Tc_ex, phc_ex, scale_T, nx, ny, nz)
ht3d_Velocity(ctx, X, Y, Z, Vx, Vy, Vz, phc_ex, scale_V, nx, ny, nz) =
    ccall((:ht3d_Velocity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Cint), ctx, X, Y, Z, Vx, Vy, Vz, phc_ex, scale_V, nx, ny, nz)
ht3d_EffectiveThermalConductivity(ctx, X, Tc_ex, phi0, phc_ex, scale_T, nx, ny, nz) =
    ccall((:ht3d_EffectiveThermalConductivity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, CuPtr{Cdouble}, Cdouble, Cint, Cint, Cint), ctx, X, Tc_ex, phi0, phc_ex, scale_T, nx, ny, nz)
ht3d_EffectiveHeatCapacity(ctx, Ceff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho, nx, ny, nz) =
    ccall((:ht3d_EffectiveHeatCapacity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, Ceff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho, nx, ny, nz)
ht3d_Permeability(ctx, X, k_fact, ymin, dy, phc_ex, delta, scale_L, nx, ny, nz) =
    ccall((:ht3d_Permeability, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint), ctx, X, k_fact, ymin, dy, phc_ex, delta, scale_L, nx, ny, nz)
ht3d_FluidDensity(ctx, X, Tc_ex, Pc_ex, phc_ex, scale_T, scale_sigma, nx, ny, nz) =
    ccall((:ht3d_FluidDensity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint), ctx, X, Tc_ex, Pc_ex, phc_ex, scale_T, scale_sigma, nx, ny, nz)
ht3d_Viscosity(ctx, X, Tc_ex, phc_ex, scale_T, nx, ny, nz) =
    ccall((:ht3d_Viscosity, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Cint), ctx, X, Tc_ex, phc_ex, scale_T, nx, ny, nz)
ht3d_Peclet(ctx, X, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, phi0, scale_T, scale_sigma, scale_V, scale_L, nx, ny, nz) =
    ccall((:ht3d_Peclet, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cint, Cint, Cint), ctx, X, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, phi0, scale_T, scale_sigma, scale_V, scale_L, nx, ny, nz)
ht3d_postprocess_fields(ctx, out, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, prm, nx, ny, nz) =
    ccall((:ht3d_postprocess_fields, libht3d), Cint, (Ptr{Cvoid}, Ref{PostFields}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ref{PostParams}, Cint, Cint, Cint), ctx, out, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, prm, nx, ny, nz)
ht3d_sizeof_post_params() =
    ccall((:ht3d_sizeof_post_params, libht3d), Cint, ())
ht3d_sizeof_post_fields() =
    ccall((:ht3d_sizeof_post_fields, libht3d), Cint, ())
ht3d_Nusselt(ctx, qy, Lx, Lz, nx, ny, nz, Nu) =
    ccall((:ht3d_Nusselt, libht3d), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint, Ptr{Cdouble}), ctx, qy, Lx, Lz, nx, ny, nz, Nu)
ht3d_write_vtr(path, x, y, z, nx, ny, nz, nfields, names, ncomp, data) =
    ccall((:ht3d_write_vtr, libht3d), Cint, (Cstring, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Cint, Cint, Cint, Ptr{Cstring}, Ptr{Cint}, Ptr{Ptr{Cdouble}}), path, x, y, z, nx, ny, nz, nfields, names, ncomp, data)
ht3d_breakpoint_write(ctx, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz) =
    ccall((:ht3d_breakpoint_write, libht3d), Cint, (Ptr{Cvoid}, Cstring, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint), ctx, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz)
ht3d_breakpoint_read(ctx, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz) =
    ccall((:ht3d_breakpoint_read, libht3d), Cint, (Ptr{Cvoid}, Cstring, CuPtr{Cdouble}, CuPtr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Cint, Cint), ctx, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz)
ht3d_breakpoint_write_h5(ctx, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz) =
    ccall((:ht3d_breakpoint_write_h5, libht3d), Cint, (Ptr{Cvoid}, Cstring, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint), ctx, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz)
ht3d_breakpoint_read_h5(ctx, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz) =
    ccall((:ht3d_breakpoint_read_h5, libht3d), Cint, (Ptr{Cvoid}, Cstring, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), ctx, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz)
ht3d_h5_breakpoint_image(path, Tc_ex, Pc_ex, time, dt, nx, ny, nz) =
    ccall((:ht3d_h5_breakpoint_image, libht3d), Cint, (Cstring, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cdouble, Cint, Cint, Cint), path, Tc_ex, Pc_ex, time, dt, nx, ny, nz)
ht3d_h5_breakpoint_parse(path, Tc_ex, Pc_ex, time, dt, nx, ny, nz) =
    ccall((:ht3d_h5_breakpoint_parse, libht3d), Cint, (Cstring, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cint, Cint, Cint), path, Tc_ex, Pc_ex, time, dt, nx, ny, nz)

end  # module C

# ---------------------------------------------------------------- context and errors
struct Ht3dError <: Exception
    status::Cint
    msg::String
end
Base.showerror(io::IO, e::Ht3dError) = print(io, "libht3d status ", e.status, " (", e.msg, ")")

mutable struct Context
    ptr::Ptr{Cvoid}
end

"""
    Context(; device = 0, stream = CUDA.stream())

One libht3d context: its CUDA stream and scratch memory.  Destroyed by the GC.
"""
function Context(; device::Integer = 0, stream = CUDA.stream())
    r = Ref{Ptr{Cvoid}}(C_NULL)
    st = C.ht3d_ctx_create(r, Cint(device), Ptr{Cvoid}(stream.handle))
    st == OK || throw(Ht3dError(st, unsafe_string(C.ht3d_status_string(st))))
    ctx = Context(r[])
    finalizer(ctx) do c
        c.ptr == C_NULL || C.ht3d_ctx_destroy(c.ptr)
        c.ptr = C_NULL
    end
    return ctx
end

const _default = Ref{Union{Nothing, Context}}(nothing)
"""The default context (created on first use on CUDA.jl's current stream)."""
context() = (_default[] === nothing && (_default[] = Context()); _default[])

function _check(ctx::Context, st::Cint)
    st == OK && return nothing
    msg = unsafe_string(C.ht3d_status_string(st))
    detail = unsafe_string(C.ht3d_ctx_last_error(ctx.ptr))
    throw(Ht3dError(st, isempty(detail) ? msg : msg * ": " * detail))
end

function _shape(a, dims, name)
    size(a) == dims || throw(ArgumentError("$name: shape $(size(a)) does not match the staggering $dims"))
    return nothing
end

function __init__()
    C.ht3d_abi_version() == ABI_VERSION || error("libht3d ABI version mismatch")
    for (T, n) in ((DyrelParams, C.ht3d_sizeof_dyrel_params()), (DyrelStats, C.ht3d_sizeof_dyrel_stats()),
                   (HrlParams, C.ht3d_sizeof_hrl_params()), (V18Params, C.ht3d_sizeof_v18_params()),
                   (Instance, C.ht3d_sizeof_instance()), (PostParams, C.ht3d_sizeof_post_params()),
                   (PostFields, C.ht3d_sizeof_post_fields()))
        sizeof(T) == n || error("libht3d struct size mismatch: $T")
    end
end

"""DYREL controls with the reference's values (Dimensional/HydroThermal3D_v18.jl:292-303, 433-439)."""
reference_dyrel(; tol = 1e-8, nitmax = 10000, nitout = 1000, norm_scale = 1.0) =
    DyrelParams(tol_abs = tol, tol_rel = tol, nitmax = Cint(nitmax), nitout = Cint(nitout), cfl = 0.99,
                cfact = 0.5, lmin_ratio = 500.0, norm_scale = norm_scale)

# ---------------------------------------------------------------- drop-in kernels
"""
    Init_vel!(Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty, Ra, _dx, _dy, _dz)

`@parallel Init_vel!(...)` of Dimensionless/kernels_HT3D.jl:73-80, on the GPU through `ht3d_Init_vel`.
"""
function Init_vel!(Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty, Ra, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(Pc_ex) .- 2
    _shape(Vx, (nx + 1, ny, nz), "Vx")
    _shape(Vy, (nx, ny + 1, nz), "Vy")
    _shape(Vz, (nx, ny, nz + 1), "Vz")
    _shape(kx, (nx + 1, ny, nz), "kx")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(kz, (nx, ny, nz + 1), "kz")
    _shape(Pc_ex, (nx + 2, ny + 2, nz + 2), "Pc_ex")
    _shape(Ty, (nx, ny + 1, nz), "Ty")
    _check(ctx, C.ht3d_Init_vel(ctx.ptr, Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty, Ra, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    InitDarcy!(Ty, kx, ky, kz, Tc_ex, kfv, _dt)

`@parallel InitDarcy!(...)` of Dimensionless/kernels_HT3D.jl:82-90, on the GPU through `ht3d_InitDarcy`.
"""
function InitDarcy!(Ty, kx, ky, kz, Tc_ex, kfv, _dt; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _shape(Ty, (nx, ny + 1, nz), "Ty")
    _shape(kx, (nx + 1, ny, nz), "kx")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(kz, (nx, ny, nz + 1), "kz")
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(kfv, (nx + 1, ny + 1, nz + 1), "kfv")
    _check(ctx, C.ht3d_InitDarcy(ctx.ptr, Ty, kx, ky, kz, Tc_ex, kfv, _dt, nx, ny, nz))
    return nothing
end

"""
    Compute_Rp!(Rp, ky, Ty, Ra, _dy)

`@parallel Compute_Rp!(...)` of Dimensionless/kernels_HT3D.jl:92-97, on the GPU through `ht3d_Compute_Rp`.
"""
function Compute_Rp!(Rp, ky, Ty, Ra, _dy; ctx::Context = context())
    nx, ny, nz = size(Rp) .- 0
    _shape(Rp, (nx, ny, nz), "Rp")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(Ty, (nx, ny + 1, nz), "Ty")
    _check(ctx, C.ht3d_Compute_Rp(ctx.ptr, Rp, ky, Ty, Ra, _dy, nx, ny, nz))
    return nothing
end

"""
    InitThermal!(Rt, kx, ky, kz, Tc_ex, ktv, _dt)

`@parallel InitThermal!(...)` of Dimensionless/kernels_HT3D.jl:99-107, on the GPU through `ht3d_InitThermal`.
"""
function InitThermal!(Rt, kx, ky, kz, Tc_ex, ktv, _dt; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _shape(Rt, (nx, ny, nz), "Rt")
    _shape(kx, (nx + 1, ny, nz), "kx")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(kz, (nx, ny, nz + 1), "kz")
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(ktv, (nx + 1, ny + 1, nz + 1), "ktv")
    _check(ctx, C.ht3d_InitThermal(ctx.ptr, Rt, kx, ky, kz, Tc_ex, ktv, _dt, nx, ny, nz))
    return nothing
end

"""
    ComputeFlux!(qx, qy, qz, kx, ky, kz, A, _dx, _dy, _dz)

`@parallel ComputeFlux!(...)` of Dimensionless/kernels_HT3D.jl:109-117, Dimensional/kernels_HT3D_dimensional.jl:140-146, on the GPU through `ht3d_ComputeFlux`.
"""
function ComputeFlux!(qx, qy, qz, kx, ky, kz, A, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(A) .- 2
    _shape(qx, (nx + 1, ny, nz), "qx")
    _shape(qy, (nx, ny + 1, nz), "qy")
    _shape(qz, (nx, ny, nz + 1), "qz")
    _shape(kx, (nx + 1, ny, nz), "kx")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(kz, (nx, ny, nz + 1), "kz")
    _shape(A, (nx + 2, ny + 2, nz + 2), "A")
    _check(ctx, C.ht3d_ComputeFlux(ctx.ptr, qx, qy, qz, kx, ky, kz, A, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    UpdateT!(F, T, R, qx, qy, qz, _dt, dtau, _dx, _dy, _dz)

`@parallel UpdateT!(...)` of Dimensionless/kernels_HT3D.jl:119-126, on the GPU through `ht3d_UpdateT`.
"""
function UpdateT!(F, T, R, qx, qy, qz, _dt, dtau, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(F) .- 0
    _shape(F, (nx, ny, nz), "F")
    _shape(T, (nx + 2, ny + 2, nz + 2), "T")
    _shape(R, (nx, ny, nz), "R")
    _shape(qx, (nx + 1, ny, nz), "qx")
    _shape(qy, (nx, ny + 1, nz), "qy")
    _shape(qz, (nx, ny, nz + 1), "qz")
    _check(ctx, C.ht3d_UpdateT(ctx.ptr, F, T, R, qx, qy, qz, _dt, dtau, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    ResidualDiffusion!(F, R, qx, qy, qz, _dx, _dy, _dz)

`@parallel ResidualDiffusion!(...)` of Dimensionless/kernels_HT3D.jl:128-134, on the GPU through `ht3d_ResidualDiffusion`.
"""
function ResidualDiffusion!(F, R, qx, qy, qz, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(F) .- 0
    _shape(F, (nx, ny, nz), "F")
    _shape(R, (nx, ny, nz), "R")
    _shape(qx, (nx + 1, ny, nz), "qx")
    _shape(qy, (nx, ny + 1, nz), "qy")
    _shape(qz, (nx, ny, nz + 1), "qz")
    _check(ctx, C.ht3d_ResidualDiffusion(ctx.ptr, F, R, qx, qy, qz, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    ResidualDiffusionTransient!(F, T, R, qx, qy, qz, _dt, _dx, _dy, _dz)

`@parallel ResidualDiffusionTransient!(...)` of Dimensionless/HydroThermal3D_Alban_v6.jl:84-90, on the GPU through `ht3d_ResidualDiffusionTransient`.
"""
function ResidualDiffusionTransient!(F, T, R, qx, qy, qz, _dt, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(F) .- 0
    _shape(F, (nx, ny, nz), "F")
    _shape(T, (nx + 2, ny + 2, nz + 2), "T")
    _shape(R, (nx, ny, nz), "R")
    _shape(qx, (nx + 1, ny, nz), "qx")
    _shape(qy, (nx, ny + 1, nz), "qy")
    _shape(qz, (nx, ny, nz + 1), "qz")
    _check(ctx, C.ht3d_ResidualDiffusionTransient(ctx.ptr, F, T, R, qx, qy, qz, _dt, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    UpdateP!(F0, P, F, dampx, dtau)

`@parallel UpdateP!(...)` of Dimensionless/kernels_HT3D.jl:136-142, on the GPU through `ht3d_UpdateP`.
"""
function UpdateP!(F0, P, F, dampx, dtau; ctx::Context = context())
    nx, ny, nz = size(F) .- 0
    _shape(F0, (nx, ny, nz), "F0")
    _shape(P, (nx + 2, ny + 2, nz + 2), "P")
    _shape(F, (nx, ny, nz), "F")
    _check(ctx, C.ht3d_UpdateP(ctx.ptr, F0, P, F, dampx, dtau, nx, ny, nz))
    return nothing
end

"""
    DampedUpdate!(F0, P, F, dampx, dtau)

`@parallel DampedUpdate!(...)` of Dimensional/kernels_HT3D_dimensional.jl:316-320, on the GPU through `ht3d_UpdateP`.
"""
function DampedUpdate!(F0, P, F, dampx, dtau; ctx::Context = context())
    nx, ny, nz = size(F) .- 0
    _shape(F0, (nx, ny, nz), "F0")
    _shape(P, (nx + 2, ny + 2, nz + 2), "P")
    _shape(F, (nx, ny, nz), "F")
    _check(ctx, C.ht3d_UpdateP(ctx.ptr, F0, P, F, dampx, dtau, nx, ny, nz))
    return nothing
end

"""
    DYRELUpdate!(F0, X, F, h1, h2, dtau)

`@parallel DYRELUpdate!(...)` of Dimensional/kernels_HT3D_dimensional.jl:322-326, on the GPU through `ht3d_DYRELUpdate`.
"""
function DYRELUpdate!(F0, X, F, h1, h2, dtau; ctx::Context = context())
    nx, ny, nz = size(F) .- 0
    _shape(F0, (nx, ny, nz), "F0")
    _shape(X, (nx + 2, ny + 2, nz + 2), "X")
    _shape(F, (nx, ny, nz), "F")
    _check(ctx, C.ht3d_DYRELUpdate(ctx.ptr, F0, X, F, h1, h2, dtau, nx, ny, nz))
    return nothing
end

"""
    SetPressureBCs!(Pc_ex, Pbot, Ptop)

`@parallel SetPressureBCs!(...)` of Dimensionless/kernels_HT3D.jl:144-154, on the GPU through `ht3d_SetPressureBCs`.
"""
function SetPressureBCs!(Pc_ex, Pbot, Ptop; ctx::Context = context())
    nx, ny, nz = size(Pc_ex) .- 2
    _check(ctx, C.ht3d_SetPressureBCs(ctx.ptr, Pc_ex, Pbot, Ptop, nx, ny, nz))
    return nothing
end

"""
    SetFaceBCs!(X_ex, bc_type6, bc_val6)

`@parallel SetFaceBCs!(...)` of the face rules of Dimensionless/HydroThermal3D_Alban_v6.jl:108-130 (faces W,E,S,N,B,F), on the GPU through `ht3d_SetFaceBCs`.
"""
function SetFaceBCs!(X_ex, bc_type6, bc_val6; ctx::Context = context())
    nx, ny, nz = size(X_ex) .- 2
    _check(ctx, C.ht3d_SetFaceBCs(ctx.ptr, X_ex, bc_type6, bc_val6, nx, ny, nz))
    return nothing
end

"""
    KillNorthSouthFluxes!(Ty)

`@parallel KillNorthSouthFluxes!(...)` of Dimensionless/HydroThermal3D_Alban_v6.jl:153-159, on the GPU through `ht3d_KillNorthSouthFluxes`.
"""
function KillNorthSouthFluxes!(Ty; ctx::Context = context())
    nx, ny, nz = size(Ty) .- (0, 1, 0)
    _check(ctx, C.ht3d_KillNorthSouthFluxes(ctx.ptr, Ty, nx, ny, nz))
    return nothing
end

"""
    ResetA!(A, B)

`@parallel ResetA!(...)` of tools/Macros.jl:171-177, on the GPU through `ht3d_ResetA`.
"""
function ResetA!(A, B; ctx::Context = context())
    _check(ctx, C.ht3d_ResetA(ctx.ptr, A, B, length(A)))
    return nothing
end

"""
    Cpy_inn_to_all!(A, B_ex)

`@parallel Cpy_inn_to_all!(...)` of tools/Macros.jl:187-192, on the GPU through `ht3d_Cpy_inn_to_all`.
"""
function Cpy_inn_to_all!(A, B_ex; ctx::Context = context())
    nx, ny, nz = size(A) .- 0
    _shape(A, (nx, ny, nz), "A")
    _check(ctx, C.ht3d_Cpy_inn_to_all(ctx.ptr, A, B_ex, nx, ny, nz))
    return nothing
end

"""
    Cpy_all_to_inn!(A_ex, B)

`@parallel Cpy_all_to_inn!(...)` of tools/Macros.jl:194-199, on the GPU through `ht3d_Cpy_all_to_inn`.
"""
function Cpy_all_to_inn!(A_ex, B; ctx::Context = context())
    nx, ny, nz = size(B) .- 0
    _shape(B, (nx, ny, nz), "B")
    _check(ctx, C.ht3d_Cpy_all_to_inn(ctx.ptr, A_ex, B, nx, ny, nz))
    return nothing
end

"""
    ArrayEqualArray!(A, B)

`@parallel ArrayEqualArray!(...)` of tools/Weno5_Routines.jl:271-276, on the GPU through `ht3d_ArrayEqualArray`.
"""
function ArrayEqualArray!(A, B; ctx::Context = context())
    _check(ctx, C.ht3d_ArrayEqualArray(ctx.ptr, A, B, length(A)))
    return nothing
end

"""
    Multiply(a, b, c)

`@parallel Multiply(...)` of Dimensional/kernels_HT3D_dimensional.jl:106-109, on the GPU through `ht3d_Multiply`.
"""
function Multiply(a, b, c; ctx::Context = context())
    _check(ctx, C.ht3d_Multiply(ctx.ptr, a, b, c, length(a)))
    return nothing
end

"""
    InitThermal!(A, B_ex)

`@parallel InitThermal!(...)` of Dimensional/kernels_HT3D_dimensional.jl:128-131, on the GPU through `ht3d_Cpy_inn_to_all`.
"""
function InitThermal!(A, B_ex; ctx::Context = context())
    nx, ny, nz = size(A) .- 0
    _shape(A, (nx, ny, nz), "A")
    _check(ctx, C.ht3d_Cpy_inn_to_all(ctx.ptr, A, B_ex, nx, ny, nz))
    return nothing
end

"""
    InitDarcy!(A, B)

`@parallel InitDarcy!(...)` of Dimensional/kernels_HT3D_dimensional.jl:261-264, on the GPU through `ht3d_ArrayEqualArray`.
"""
function InitDarcy!(A, B; ctx::Context = context())
    _check(ctx, C.ht3d_ArrayEqualArray(ctx.ptr, A, B, length(A)))
    return nothing
end

"""
    GershgorinPoisson!(G, D, rhoC_eff, kx, ky, kz, transient, dt, dx, dy, dz)

`@parallel GershgorinPoisson!(...)` of Dimensional/kernels_HT3D_dimensional.jl:207-221, on the GPU through `ht3d_GershgorinPoisson`.
"""
function GershgorinPoisson!(G, D, rhoC_eff, kx, ky, kz, transient, dt, dx, dy, dz; ctx::Context = context())
    nx, ny, nz = size(G) .- 0
    _shape(G, (nx, ny, nz), "G")
    _shape(D, (nx, ny, nz), "D")
    _shape(rhoC_eff, (nx, ny, nz), "rhoC_eff")
    _shape(kx, (nx + 1, ny, nz), "kx")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(kz, (nx, ny, nz + 1), "kz")
    _check(ctx, C.ht3d_GershgorinPoisson(ctx.ptr, G, D, rhoC_eff, kx, ky, kz, transient, dt, dx, dy, dz, nx, ny, nz))
    return nothing
end

"""
    GershgorinHydro!(G, phidrhodP, kx, ky, kz, transient, dt, dx, dy, dz)

`@parallel GershgorinHydro!(...)` of Dimensional/kernels_HT3D_dimensional.jl:335-347, on the GPU through `ht3d_GershgorinHydro`.
"""
function GershgorinHydro!(G, phidrhodP, kx, ky, kz, transient, dt, dx, dy, dz; ctx::Context = context())
    nx, ny, nz = size(G) .- 0
    _shape(G, (nx, ny, nz), "G")
    _shape(phidrhodP, (nx, ny, nz), "phidrhodP")
    _shape(kx, (nx + 1, ny, nz), "kx")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(kz, (nx, ny, nz + 1), "kz")
    _check(ctx, C.ht3d_GershgorinHydro(ctx.ptr, G, phidrhodP, kx, ky, kz, transient, dt, dx, dy, dz, nx, ny, nz))
    return nothing
end

"""
    SwapDYREL!(Xc, Yc, X0c_ex, Y0c)

`@parallel SwapDYREL!(...)` of Dimensional/kernels_HT3D_dimensional.jl:122-126, on the GPU through `ht3d_SwapDYREL`.
"""
function SwapDYREL!(Xc, Yc, X0c_ex, Y0c; ctx::Context = context())
    nx, ny, nz = size(Xc) .- 0
    _shape(Xc, (nx, ny, nz), "Xc")
    _shape(Yc, (nx, ny, nz), "Yc")
    _shape(X0c_ex, (nx + 2, ny + 2, nz + 2), "X0c_ex")
    _shape(Y0c, (nx, ny, nz), "Y0c")
    _check(ctx, C.ht3d_SwapDYREL(ctx.ptr, Xc, Yc, X0c_ex, Y0c, nx, ny, nz))
    return nothing
end

"""
    RayleighQuotientNumerator!(G, Fc0, Fcit, Fc, dtau)

`@parallel RayleighQuotientNumerator!(...)` of Dimensional/kernels_HT3D_dimensional.jl:349-355, on the GPU through `ht3d_RayleighQuotientNumerator`.
"""
function RayleighQuotientNumerator!(G, Fc0, Fcit, Fc, dtau; ctx::Context = context())
    _check(ctx, C.ht3d_RayleighQuotientNumerator(ctx.ptr, G, Fc0, Fcit, Fc, dtau, length(G)))
    return nothing
end

"""
    RayleighQuotientDenominator!(G, Fc0, dtau)

`@parallel RayleighQuotientDenominator!(...)` of Dimensional/kernels_HT3D_dimensional.jl:357-363, on the GPU through `ht3d_RayleighQuotientDenominator`.
"""
function RayleighQuotientDenominator!(G, Fc0, dtau; ctx::Context = context())
    _check(ctx, C.ht3d_RayleighQuotientDenominator(ctx.ptr, G, Fc0, dtau, length(G)))
    return nothing
end

"""
    ComputeThermalConductivity(ktv, Tce, phv, phi0, scale_kt, scale_T)

`@parallel ComputeThermalConductivity(...)` of Dimensional/kernels_HT3D_dimensional.jl:40-50, on the GPU through `ht3d_ComputeThermalConductivity`.
"""
function ComputeThermalConductivity(ktv, Tce, phv, phi0, scale_kt, scale_T; ctx::Context = context())
    nx, ny, nz = size(ktv) .- 1
    _shape(ktv, (nx + 1, ny + 1, nz + 1), "ktv")
    _shape(Tce, (nx + 2, ny + 2, nz + 2), "Tce")
    _shape(phv, (nx + 1, ny + 1, nz + 1), "phv")
    _check(ctx, C.ht3d_ComputeThermalConductivity(ctx.ptr, ktv, Tce, phv, phi0, scale_kt, scale_T, nx, ny, nz))
    return nothing
end

"""
    ComputeHydroConductivity(kfv, Tce, Pce, phv, ymin, dy, k_fact, delta, scale_sigma, scale_T, scale_L, scale_t, scale_eta, mode)

`@parallel ComputeHydroConductivity(...)` of Dimensional/kernels_HT3D_dimensional.jl:52-86, on the GPU through `ht3d_ComputeHydroConductivity`.
"""
function ComputeHydroConductivity(kfv, Tce, Pce, phv, ymin, dy, k_fact, delta, scale_sigma, scale_T, scale_L, scale_t, scale_eta, mode; kmul_v = CU_NULL, ctx::Context = context())
    nx, ny, nz = size(kfv) .- 1
    _shape(kfv, (nx + 1, ny + 1, nz + 1), "kfv")
    _shape(Tce, (nx + 2, ny + 2, nz + 2), "Tce")
    _shape(Pce, (nx + 2, ny + 2, nz + 2), "Pce")
    _shape(phv, (nx + 1, ny + 1, nz + 1), "phv")
    _check(ctx, C.ht3d_ComputeHydroConductivity(ctx.ptr, kfv, Tce, Pce, phv, ymin, dy, k_fact, delta, scale_sigma, scale_T, scale_L, scale_t, scale_eta, mode, kmul_v, nx, ny, nz))
    return nothing
end

"""
    ComputeFluidDensity(rhofv, Tce, Pce, phv, scale_sigma, scale_T, scale_rho)

`@parallel ComputeFluidDensity(...)` of Dimensional/kernels_HT3D_dimensional.jl:88-104, on the GPU through `ht3d_ComputeFluidDensity`.
"""
function ComputeFluidDensity(rhofv, Tce, Pce, phv, scale_sigma, scale_T, scale_rho; ctx::Context = context())
    nx, ny, nz = size(rhofv) .- 1
    _shape(rhofv, (nx + 1, ny + 1, nz + 1), "rhofv")
    _shape(Tce, (nx + 2, ny + 2, nz + 2), "Tce")
    _shape(Pce, (nx + 2, ny + 2, nz + 2), "Pce")
    _shape(phv, (nx + 1, ny + 1, nz + 1), "phv")
    _check(ctx, C.ht3d_ComputeFluidDensity(ctx.ptr, rhofv, Tce, Pce, phv, scale_sigma, scale_T, scale_rho, nx, ny, nz))
    return nothing
end

"""
    SmoothConductivityV2C(ktc, ktv)

`@parallel SmoothConductivityV2C(...)` of Dimensional/kernels_HT3D_dimensional.jl:111-114, on the GPU through `ht3d_SmoothConductivityV2C`.
"""
function SmoothConductivityV2C(ktc, ktv; ctx::Context = context())
    nx, ny, nz = size(ktc) .- 0
    _shape(ktv, (nx + 2, nz + 2), "ktv")
    _check(ctx, C.ht3d_SmoothConductivityV2C(ctx.ptr, ktc, ktv, nx, ny, nz))
    return nothing
end

"""
    SmoothConductivityC2V(ktv, ktc)

`@parallel SmoothConductivityC2V(...)` of Dimensional/kernels_HT3D_dimensional.jl:116-119, on the GPU through `ht3d_SmoothConductivityC2V`.
"""
function SmoothConductivityC2V(ktv, ktc; ctx::Context = context())
    nx, ny, nz = size(ktc) .- 0
    _shape(ktv, (nx + 2, nz + 2), "ktv")
    _check(ctx, C.ht3d_SmoothConductivityC2V(ctx.ptr, ktv, ktc, nx, ny, nz))
    return nothing
end

"""
    InitConductivity!(kx, ky, kz, ktv)

`@parallel InitConductivity!(...)` of Dimensional/kernels_HT3D_dimensional.jl:133-138, on the GPU through `ht3d_InitConductivity`.
"""
function InitConductivity!(kx, ky, kz, ktv; ctx::Context = context())
    nx, ny, nz = size(ktv) .- 1
    _shape(kx, (nx + 1, ny, nz), "kx")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(kz, (nx, ny, nz + 1), "kz")
    _check(ctx, C.ht3d_InitConductivity(ctx.ptr, kx, ky, kz, ktv, nx, ny, nz))
    return nothing
end

"""
    ComputeρCeffective!(rhoC_eff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho)

`@parallel ComputeρCeffective!(...)` of Dimensional/kernels_HT3D_dimensional.jl:148-160, on the GPU through `ht3d_ComputeRhoCeffective`.
"""
function ComputeρCeffective!(rhoC_eff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho; ctx::Context = context())
    nx, ny, nz = size(rhoC_eff) .- 0
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(Pc_ex, (nx + 2, ny + 2, nz + 2), "Pc_ex")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_ComputeRhoCeffective(ctx.ptr, rhoC_eff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho, nx, ny, nz))
    return nothing
end

"""
    ResidualTemperatureLinearised!(F, Tc_ex, Tc_old, rhoC_eff, phc_ex, PC, qx, qy, qz, Qt, transient, _dt, _dx, _dy, _dz)

`@parallel ResidualTemperatureLinearised!(...)` of Dimensional/kernels_HT3D_dimensional.jl:162-181, on the GPU through `ht3d_ResidualTemperatureLinearised`.
"""
function ResidualTemperatureLinearised!(F, Tc_ex, Tc_old, rhoC_eff, phc_ex, PC, qx, qy, qz, Qt, transient, _dt, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(F) .- 0
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(Tc_old, (nx, ny, nz), "Tc_old")
    _shape(rhoC_eff, (nx, ny, nz), "rhoC_eff")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _shape(PC, (nx, ny, nz), "PC")
    _shape(qx, (nx + 1, ny, nz), "qx")
    _shape(qy, (nx, ny + 1, nz), "qy")
    _shape(qz, (nx, ny, nz + 1), "qz")
    _check(ctx, C.ht3d_ResidualTemperatureLinearised(ctx.ptr, F, Tc_ex, Tc_old, rhoC_eff, phc_ex, PC, qx, qy, qz, Qt, transient, _dt, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    SetTemperatureBCs!(Tc_ex, ky, wN, phc_ex, qyS, _dy, kS, TS, TN, y_plateau, a2, b2, dTdy, dx, dy, sticky_air, sca_T, sca_kT, phi_i)

`@parallel SetTemperatureBCs!(...)` of Dimensional/kernels_HT3D_dimensional.jl:183-205, on the GPU through `ht3d_SetTemperatureBCs`.
"""
function SetTemperatureBCs!(Tc_ex, ky, wN, phc_ex, qyS, _dy, kS, TS, TN, y_plateau, a2, b2, dTdy, dx, dy, sticky_air, sca_T, sca_kT, phi_i; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(wN, (nx + 2, nz + 2), "wN")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_SetTemperatureBCs(ctx.ptr, Tc_ex, ky, wN, phc_ex, qyS, _dy, kS, TS, TN, y_plateau, a2, b2, dTdy, dx, dy, sticky_air, sca_T, sca_kT, phi_i, nx, ny, nz))
    return nothing
end

"""
    SetPressureBCs!(Pc_ex, wN, phc_ex, PS, PN, y_plateau, a2, b2, rhof, g, dx, dy, sticky_air)

`@parallel SetPressureBCs!(...)` of Dimensional/kernels_HT3D_dimensional.jl:291-314, on the GPU through `ht3d_SetPressureBCs_dim`.
"""
function SetPressureBCs!(Pc_ex, wN, phc_ex, PS, PN, y_plateau, a2, b2, rhof, g, dx, dy, sticky_air; ctx::Context = context())
    nx, ny, nz = size(Pc_ex) .- 2
    _shape(wN, (nx + 2, nz + 2), "wN")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_SetPressureBCs_dim(ctx.ptr, Pc_ex, wN, phc_ex, PS, PN, y_plateau, a2, b2, rhof, g, dx, dy, sticky_air, nx, ny, nz))
    return nothing
end

"""
    ϕρf(phirhofc, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma)

`@parallel ϕρf(...)` of Dimensional/kernels_HT3D_dimensional.jl:225-235, on the GPU through `ht3d_PhiRhof`.
"""
function ϕρf(phirhofc, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma; ctx::Context = context())
    nx, ny, nz = size(phirhofc) .- 0
    _check(ctx, C.ht3d_PhiRhof(ctx.ptr, phirhofc, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz))
    return nothing
end

"""
    ϕρf_old(phirhofc, Tc0, Pc0, phc_ex, phi_i, scale_rho, scale_T, scale_sigma)

`@parallel ϕρf_old(...)` of Dimensional/kernels_HT3D_dimensional.jl:237-247, on the GPU through `ht3d_PhiRhofOld`.
"""
function ϕρf_old(phirhofc, Tc0, Pc0, phc_ex, phi_i, scale_rho, scale_T, scale_sigma; ctx::Context = context())
    nx, ny, nz = size(phirhofc) .- 0
    _check(ctx, C.ht3d_PhiRhofOld(ctx.ptr, phirhofc, Tc0, Pc0, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz))
    return nothing
end

"""
    ϕdρdP!(phidrhodP, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma)

`@parallel ϕdρdP!(...)` of Dimensional/kernels_HT3D_dimensional.jl:249-259, on the GPU through `ht3d_PhiDrhodP`.
"""
function ϕdρdP!(phidrhodP, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma; ctx::Context = context())
    nx, ny, nz = size(phidrhodP) .- 0
    _check(ctx, C.ht3d_PhiDrhodP(ctx.ptr, phidrhodP, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma, nx, ny, nz))
    return nothing
end

"""
    ComputeDarcyFlux!(qx, qy, qz, rhofv, kx, ky, kz, Pf, g, _dx, _dy, _dz)

`@parallel ComputeDarcyFlux!(...)` of Dimensional/kernels_HT3D_dimensional.jl:266-272, on the GPU through `ht3d_ComputeDarcyFlux`.
"""
function ComputeDarcyFlux!(qx, qy, qz, rhofv, kx, ky, kz, Pf, g, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(Pf) .- 2
    _shape(qx, (nx + 1, ny, nz), "qx")
    _shape(qy, (nx, ny + 1, nz), "qy")
    _shape(qz, (nx, ny, nz + 1), "qz")
    _shape(rhofv, (nx + 1, ny + 1, nz + 1), "rhofv")
    _shape(kx, (nx + 1, ny, nz), "kx")
    _shape(ky, (nx, ny + 1, nz), "ky")
    _shape(kz, (nx, ny, nz + 1), "kz")
    _shape(Pf, (nx + 2, ny + 2, nz + 2), "Pf")
    _check(ctx, C.ht3d_ComputeDarcyFlux(ctx.ptr, qx, qy, qz, rhofv, kx, ky, kz, Pf, g, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    ResidualFluidPressure!(F, phc_ex, phirhofc, phirhofc0, PC, qx, qy, qz, transient, _dt, _dx, _dy, _dz)

`@parallel ResidualFluidPressure!(...)` of Dimensional/kernels_HT3D_dimensional.jl:274-289, on the GPU through `ht3d_ResidualFluidPressure`.
"""
function ResidualFluidPressure!(F, phc_ex, phirhofc, phirhofc0, PC, qx, qy, qz, transient, _dt, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(F) .- 0
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _shape(phirhofc, (nx, ny, nz), "phirhofc")
    _shape(phirhofc0, (nx, ny, nz), "phirhofc0")
    _shape(PC, (nx, ny, nz), "PC")
    _shape(qx, (nx + 1, ny, nz), "qx")
    _shape(qy, (nx, ny + 1, nz), "qy")
    _shape(qz, (nx, ny, nz + 1), "qz")
    _check(ctx, C.ht3d_ResidualFluidPressure(ctx.ptr, F, phc_ex, phirhofc, phirhofc0, PC, qx, qy, qz, transient, _dt, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    Init_vel!(Vx, Vy, Vz, qx, qy, qz, rhofv)

`@parallel Init_vel!(...)` of Dimensional/kernels_HT3D_dimensional.jl:328-333, on the GPU through `ht3d_Init_vel_dim`.
"""
function Init_vel!(Vx, Vy, Vz, qx, qy, qz, rhofv; ctx::Context = context())
    nx, ny, nz = size(rhofv) .- 1
    _shape(Vx, (nx + 1, ny, nz), "Vx")
    _shape(Vy, (nx, ny + 1, nz), "Vy")
    _shape(Vz, (nx, ny, nz + 1), "Vz")
    _shape(qx, (nx + 1, ny, nz), "qx")
    _shape(qy, (nx, ny + 1, nz), "qy")
    _shape(qz, (nx, ny, nz + 1), "qz")
    _shape(rhofv, (nx + 1, ny + 1, nz + 1), "rhofv")
    _check(ctx, C.ht3d_Init_vel_dim(ctx.ptr, Vx, Vy, Vz, qx, qy, qz, rhofv, nx, ny, nz))
    return nothing
end

"""
    VxPlusMinus!(Vm, Vp, V)

`@parallel VxPlusMinus!(...)` of tools/Weno5_Routines.jl:5-16, on the GPU through `ht3d_VPlusMinus`.
"""
function VxPlusMinus!(Vm, Vp, V; ctx::Context = context())
    nx, ny, nz = size(Vm) .- 0
    _check(ctx, C.ht3d_VPlusMinus(ctx.ptr, Vm, Vp, V, 0, nx, ny, nz))
    return nothing
end

"""
    VyPlusMinus!(Vm, Vp, V)

`@parallel VyPlusMinus!(...)` of tools/Weno5_Routines.jl:18-29, on the GPU through `ht3d_VPlusMinus`.
"""
function VyPlusMinus!(Vm, Vp, V; ctx::Context = context())
    nx, ny, nz = size(Vm) .- 0
    _check(ctx, C.ht3d_VPlusMinus(ctx.ptr, Vm, Vp, V, 1, nx, ny, nz))
    return nothing
end

"""
    VzPlusMinus!(Vm, Vp, V)

`@parallel VzPlusMinus!(...)` of tools/Weno5_Routines.jl:31-42, on the GPU through `ht3d_VPlusMinus`.
"""
function VzPlusMinus!(Vm, Vp, V; ctx::Context = context())
    nx, ny, nz = size(Vm) .- 0
    _check(ctx, C.ht3d_VPlusMinus(ctx.ptr, Vm, Vp, V, 2, nx, ny, nz))
    return nothing
end

"""
    dFdx_Weno5!(dFdxi, V1, V2, V3, V4, V5)

`@parallel dFdx_Weno5!(...)` of tools/Weno5_Routines.jl:44-68, on the GPU through `ht3d_dFdx_Weno5`.
"""
function dFdx_Weno5!(dFdxi, V1, V2, V3, V4, V5; ctx::Context = context())
    _check(ctx, C.ht3d_dFdx_Weno5(ctx.ptr, dFdxi, V1, V2, V3, V4, V5, length(dFdxi)))
    return nothing
end

"""
    Gradients_minus_x_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz)

`@parallel Gradients_minus_x_Weno5!(...)` of tools/Weno5_Routines.jl:70-78, on the GPU through `ht3d_Gradients_Weno5`.
"""
function Gradients_minus_x_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(v1) .- 0
    _shape(Fc_exxx, (nx + 6, ny + 6, nz + 6), "Fc_exxx")
    _check(ctx, C.ht3d_Gradients_Weno5(ctx.ptr, v1, v2, v3, v4, v5, Fc_exxx, 0, -1, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    Gradients_plus_x_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz)

`@parallel Gradients_plus_x_Weno5!(...)` of tools/Weno5_Routines.jl:80-88, on the GPU through `ht3d_Gradients_Weno5`.
"""
function Gradients_plus_x_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(v1) .- 0
    _shape(Fc_exxx, (nx + 6, ny + 6, nz + 6), "Fc_exxx")
    _check(ctx, C.ht3d_Gradients_Weno5(ctx.ptr, v1, v2, v3, v4, v5, Fc_exxx, 0, 1, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    Gradients_minus_y_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz)

`@parallel Gradients_minus_y_Weno5!(...)` of tools/Weno5_Routines.jl:90-98, on the GPU through `ht3d_Gradients_Weno5`.
"""
function Gradients_minus_y_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(v1) .- 0
    _shape(Fc_exxx, (nx + 6, ny + 6, nz + 6), "Fc_exxx")
    _check(ctx, C.ht3d_Gradients_Weno5(ctx.ptr, v1, v2, v3, v4, v5, Fc_exxx, 1, -1, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    Gradients_plus_y_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz)

`@parallel Gradients_plus_y_Weno5!(...)` of tools/Weno5_Routines.jl:100-108, on the GPU through `ht3d_Gradients_Weno5`.
"""
function Gradients_plus_y_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(v1) .- 0
    _shape(Fc_exxx, (nx + 6, ny + 6, nz + 6), "Fc_exxx")
    _check(ctx, C.ht3d_Gradients_Weno5(ctx.ptr, v1, v2, v3, v4, v5, Fc_exxx, 1, 1, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    Gradients_minus_z_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz)

`@parallel Gradients_minus_z_Weno5!(...)` of tools/Weno5_Routines.jl:110-118, on the GPU through `ht3d_Gradients_Weno5`.
"""
function Gradients_minus_z_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(v1) .- 0
    _shape(Fc_exxx, (nx + 6, ny + 6, nz + 6), "Fc_exxx")
    _check(ctx, C.ht3d_Gradients_Weno5(ctx.ptr, v1, v2, v3, v4, v5, Fc_exxx, 2, -1, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    Gradients_plus_z_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz)

`@parallel Gradients_plus_z_Weno5!(...)` of tools/Weno5_Routines.jl:120-128, on the GPU through `ht3d_Gradients_Weno5`.
"""
function Gradients_plus_z_Weno5!(v1, v2, v3, v4, v5, Fc_exxx, _dx, _dy, _dz; ctx::Context = context())
    nx, ny, nz = size(v1) .- 0
    _shape(Fc_exxx, (nx + 6, ny + 6, nz + 6), "Fc_exxx")
    _check(ctx, C.ht3d_Gradients_Weno5(ctx.ptr, v1, v2, v3, v4, v5, Fc_exxx, 2, 1, _dx, _dy, _dz, nx, ny, nz))
    return nothing
end

"""
    Boundaries_x_Weno5!(Fc_exxx, Fc, type_L, val_L, type_R, val_R)

`@parallel Boundaries_x_Weno5!(...)` of tools/Weno5_Routines.jl:130-170, tools/Weno5_Routines_v2.jl:221-262, on the GPU through `ht3d_Boundaries_Weno5`.
"""
function Boundaries_x_Weno5!(Fc_exxx, Fc, type_L, val_L, type_R, val_R; ctx::Context = context())
    nx, ny, nz = size(Fc_exxx) .- 6
    _check(ctx, C.ht3d_Boundaries_Weno5(ctx.ptr, Fc_exxx, Fc, 0, type_L, val_L, type_R, val_R, Cint(size(Fc) == (nx + 2, ny + 2, nz + 2)), nx, ny, nz))
    return nothing
end

"""
    Boundaries_y_Weno5!(Fc_exxx, Fc, type_L, val_L, type_R, val_R)

`@parallel Boundaries_y_Weno5!(...)` of tools/Weno5_Routines.jl:172-212, tools/Weno5_Routines_v2.jl:264-304, on the GPU through `ht3d_Boundaries_Weno5`.
"""
function Boundaries_y_Weno5!(Fc_exxx, Fc, type_L, val_L, type_R, val_R; ctx::Context = context())
    nx, ny, nz = size(Fc_exxx) .- 6
    _check(ctx, C.ht3d_Boundaries_Weno5(ctx.ptr, Fc_exxx, Fc, 1, type_L, val_L, type_R, val_R, Cint(size(Fc) == (nx + 2, ny + 2, nz + 2)), nx, ny, nz))
    return nothing
end

"""
    Boundaries_z_Weno5!(Fc_exxx, Fc, type_L, val_L, type_R, val_R)

`@parallel Boundaries_z_Weno5!(...)` of tools/Weno5_Routines.jl:214-255, tools/Weno5_Routines_v2.jl:306-347, on the GPU through `ht3d_Boundaries_Weno5`.
"""
function Boundaries_z_Weno5!(Fc_exxx, Fc, type_L, val_L, type_R, val_R; ctx::Context = context())
    nx, ny, nz = size(Fc_exxx) .- 6
    _check(ctx, C.ht3d_Boundaries_Weno5(ctx.ptr, Fc_exxx, Fc, 2, type_L, val_L, type_R, val_R, Cint(size(Fc) == (nx + 2, ny + 2, nz + 2)), nx, ny, nz))
    return nothing
end

"""
    Advect!(Fc, Vxp, dTdxm, Vxm, dTdxp, dt)

`@parallel Advect!(...)` of tools/Weno5_Routines.jl:257-262, on the GPU through `ht3d_Advect_v1`.
"""
function Advect!(Fc, Vxp, dTdxm, Vxm, dTdxp, dt; ctx::Context = context())
    _check(ctx, C.ht3d_Advect_v1(ctx.ptr, Fc, Vxp, dTdxm, Vxm, dTdxp, dt, length(Fc)))
    return nothing
end

"""
    Advect!(Fc_ex, X_exxx, V, axis, dt, _dx, _dy, _dz)

`@parallel Advect!(...)` of tools/Weno5_Routines_v2.jl:55-212, on the GPU through `ht3d_Advect_v2`.
"""
function Advect!(Fc_ex, X_exxx, V, axis, dt, _dx, _dy, _dz; quirk = 1, ctx::Context = context())
    nx, ny, nz = size(Fc_ex) .- 2
    _check(ctx, C.ht3d_Advect_v2(ctx.ptr, Fc_ex, X_exxx, V, Cint(axis - 1), dt, _dx, _dy, _dz, Cint(quirk), nx, ny, nz))
    return nothing
end

"""
    Phase!(X, phc_ex)

`@parallel Phase!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:1-10, on the GPU through `ht3d_Phase`.
"""
function Phase!(X, phc_ex; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_Phase(ctx.ptr, X, phc_ex, nx, ny, nz))
    return nothing
end

"""
    Pressure!(X, Pc_ex, phc_ex, scale_sigma)

`@parallel Pressure!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:12-21, on the GPU through `ht3d_Pressure`.
"""
function Pressure!(X, Pc_ex, phc_ex, scale_sigma; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(Pc_ex, (nx + 2, ny + 2, nz + 2), "Pc_ex")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_Pressure(ctx.ptr, X, Pc_ex, phc_ex, scale_sigma, nx, ny, nz))
    return nothing
end

"""
    Temperature!(X, Tc_ex, phc_ex, scale_T)

`@parallel Temperature!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:23-32, on the GPU through `ht3d_Temperature`.
"""
function Temperature!(X, Tc_ex, phc_ex, scale_T; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_Temperature(ctx.ptr, X, Tc_ex, phc_ex, scale_T, nx, ny, nz))
    return nothing
end

"""
    Velocity!(X, Y, Z, Vx, Vy, Vz, phc_ex, scale_V)

`@parallel Velocity!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:34-45, on the GPU through `ht3d_Velocity`.
"""
function Velocity!(X, Y, Z, Vx, Vy, Vz, phc_ex, scale_V; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(Y, (nx, ny, nz), "Y")
    _shape(Z, (nx, ny, nz), "Z")
    _shape(Vx, (nx + 1, ny, nz), "Vx")
    _shape(Vy, (nx, ny + 1, nz), "Vy")
    _shape(Vz, (nx, ny, nz + 1), "Vz")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_Velocity(ctx.ptr, X, Y, Z, Vx, Vy, Vz, phc_ex, scale_V, nx, ny, nz))
    return nothing
end

"""
    EffectiveThermalConductivity!(X, Tc_ex, phi0, phc_ex, scale_T)

`@parallel EffectiveThermalConductivity!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:47-57, on the GPU through `ht3d_EffectiveThermalConductivity`.
"""
function EffectiveThermalConductivity!(X, Tc_ex, phi0, phc_ex, scale_T; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_EffectiveThermalConductivity(ctx.ptr, X, Tc_ex, phi0, phc_ex, scale_T, nx, ny, nz))
    return nothing
end

"""
    EffectiveHeatCapacity!(Ceff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho)

`@parallel EffectiveHeatCapacity!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:60-70, on the GPU through `ht3d_EffectiveHeatCapacity`.
"""
function EffectiveHeatCapacity!(Ceff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho; ctx::Context = context())
    nx, ny, nz = size(Ceff) .- 0
    _shape(Ceff, (nx, ny, nz), "Ceff")
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_EffectiveHeatCapacity(ctx.ptr, Ceff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho, nx, ny, nz))
    return nothing
end

"""
    Permeability!(X, k_fact, ymin, dy, phc_ex, delta, scale_L)

`@parallel Permeability!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:72-85, on the GPU through `ht3d_Permeability`.
"""
function Permeability!(X, k_fact, ymin, dy, phc_ex, delta, scale_L; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_Permeability(ctx.ptr, X, k_fact, ymin, dy, phc_ex, delta, scale_L, nx, ny, nz))
    return nothing
end

"""
    FluidDensity!(X, Tc_ex, Pc_ex, phc_ex, scale_T, scale_sigma)

`@parallel FluidDensity!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:87-98, on the GPU through `ht3d_FluidDensity`.
"""
function FluidDensity!(X, Tc_ex, Pc_ex, phc_ex, scale_T, scale_sigma; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(Pc_ex, (nx + 2, ny + 2, nz + 2), "Pc_ex")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_FluidDensity(ctx.ptr, X, Tc_ex, Pc_ex, phc_ex, scale_T, scale_sigma, nx, ny, nz))
    return nothing
end

"""
    Viscosity!(X, Tc_ex, phc_ex, scale_T)

`@parallel Viscosity!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:100-109, on the GPU through `ht3d_Viscosity`.
"""
function Viscosity!(X, Tc_ex, phc_ex, scale_T; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_Viscosity(ctx.ptr, X, Tc_ex, phc_ex, scale_T, nx, ny, nz))
    return nothing
end

"""
    Peclet!(X, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, phi0, scale_T, scale_sigma, scale_V, scale_L)

`@parallel Peclet!(...)` of Dimensional/kernels_HT3D_postprocessing.jl:111-129, on the GPU through `ht3d_Peclet`.
"""
function Peclet!(X, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, phi0, scale_T, scale_sigma, scale_V, scale_L; ctx::Context = context())
    nx, ny, nz = size(X) .- 0
    _shape(X, (nx, ny, nz), "X")
    _shape(Tc_ex, (nx + 2, ny + 2, nz + 2), "Tc_ex")
    _shape(Pc_ex, (nx + 2, ny + 2, nz + 2), "Pc_ex")
    _shape(Vx, (nx + 1, ny, nz), "Vx")
    _shape(Vy, (nx, ny + 1, nz), "Vy")
    _shape(Vz, (nx, ny, nz + 1), "Vz")
    _shape(phc_ex, (nx + 2, ny + 2, nz + 2), "phc_ex")
    _check(ctx, C.ht3d_Peclet(ctx.ptr, X, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, phi0, scale_T, scale_sigma, scale_V, scale_L, nx, ny, nz))
    return nothing
end

"""
    TimeAveraging!(Fc, Fold, order)

`@parallel TimeAveraging!(...)`: tools/Weno5_Routines.jl:264-269 (Fc and Fold of
one shape) or tools/Weno5_Routines_v2.jl:214-219 (Fc ghosted, Fold n^3).
"""
function TimeAveraging!(Fc, Fold, order; ctx::Context = context())
    if size(Fc) == size(Fold)
        _check(ctx, C.ht3d_TimeAveraging_v1(ctx.ptr, Fc, Fold, order, length(Fc)))
    else
        nx, ny, nz = size(Fold)
        _shape(Fc, (nx + 2, ny + 2, nz + 2), "Fc")
        _check(ctx, C.ht3d_TimeAveraging_v2(ctx.ptr, Fc, Fold, order, nx, ny, nz))
    end
    return nothing
end

"""
    maximum_g(A), minimum_g(A), sum_g(A), mean_g(A), mean_abs_g(A)

tools/Macros.jl:20-25 and mean_g(abs.(F)) (Dimensional/HydroThermal3D_v18.jl:460):
reductions in the library's canonical tree order, result on the host.
"""
function _reduce(A, op; ctx::Context = context())
    out = Ref{Cdouble}(0.0)
    _check(ctx, C.ht3d_reduce(ctx.ptr, A, length(A), Cint(op), out))
    return out[]
end
sum_g(A; kw...) = _reduce(A, 0; kw...)
maximum_g(A; kw...) = _reduce(A, 2; kw...)
minimum_g(A; kw...) = _reduce(A, 3; kw...)
mean_g(A; kw...) = sum_g(A; kw...) / length(A)
mean_abs_g(A; kw...) = _reduce(A, 1; kw...) / length(A)

# ---------------------------------------------------------------- fused entry points
"""
    dyrel_solve_dimless!(X_ex, R, kx, ky, kz, cX, dx, dy, dz, bc_type6, bc_val6, prm, n_iter_fixed, F, F0, precision)

`ht3d_dyrel_solve_dimless` (include/ht3d.h); returns stats.
"""
function dyrel_solve_dimless!(X_ex, R, kx, ky, kz, cX, dx, dy, dz, bc_type6, bc_val6, prm, n_iter_fixed, F, F0, precision; ctx::Context = context())
    nx, ny, nz = size(X_ex) .- 2
    stats = Ref{DyrelStats}()
    _check(ctx, C.ht3d_dyrel_solve_dimless(ctx.ptr, X_ex, R, kx, ky, kz, cX, dx, dy, dz, Cint[bc_type6...], Cdouble[bc_val6...], prm, n_iter_fixed, F, F0, precision, stats, nx, ny, nz))
    return stats[]
end

"""
    dyrel_iterate!(X_ex, R, kx, ky, kz, PC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter)

`ht3d_dyrel_iterate` (include/ht3d.h).
"""
function dyrel_iterate!(X_ex, R, kx, ky, kz, PC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter; ctx::Context = context())
    nx, ny, nz = size(X_ex) .- 2
    _check(ctx, C.ht3d_dyrel_iterate(ctx.ptr, X_ex, R, kx, ky, kz, PC, F0, cX, dx, dy, dz, Cint[bc_type6...], Cdouble[bc_val6...], h1, h2, dtau, n_iter, nx, ny, nz))
    return nothing
end

"""
    dyrel_thermal_iterate!(n_iter, T_ex, Rt, kx, ky, kz, PC, F0, _dt, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau)

`ht3d_dyrel_thermal_iterate` (include/ht3d.h).
"""
function dyrel_thermal_iterate!(n_iter, T_ex, Rt, kx, ky, kz, PC, F0, _dt, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau; ctx::Context = context())
    nx, ny, nz = size(T_ex) .- 2
    _check(ctx, C.ht3d_dyrel_thermal_iterate(ctx.ptr, n_iter, T_ex, Rt, kx, ky, kz, PC, F0, _dt, dx, dy, dz, Cint[bc_type6...], Cdouble[bc_val6...], h1, h2, dtau, nx, ny, nz))
    return nothing
end

"""
    dyrel_darcy_iterate!(n_iter, P_ex, Rp, kx, ky, kz, PC, F0, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau)

`ht3d_dyrel_darcy_iterate` (include/ht3d.h).
"""
function dyrel_darcy_iterate!(n_iter, P_ex, Rp, kx, ky, kz, PC, F0, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau; ctx::Context = context())
    nx, ny, nz = size(P_ex) .- 2
    _check(ctx, C.ht3d_dyrel_darcy_iterate(ctx.ptr, n_iter, P_ex, Rp, kx, ky, kz, PC, F0, dx, dy, dz, Cint[bc_type6...], Cdouble[bc_val6...], h1, h2, dtau, nx, ny, nz))
    return nothing
end

"""
    dyrel_iterate_f32!(X_ex, R, kx, ky, kz, invPC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter)

`ht3d_dyrel_iterate_f32` (include/ht3d.h).
"""
function dyrel_iterate_f32!(X_ex, R, kx, ky, kz, invPC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2, dtau, n_iter; ctx::Context = context())
    nx, ny, nz = size(X_ex) .- 2
    _check(ctx, C.ht3d_dyrel_iterate_f32(ctx.ptr, X_ex, R, kx, ky, kz, invPC, F0, cX, dx, dy, dz, Cint[bc_type6...], Cdouble[bc_val6...], h1, h2, dtau, n_iter, nx, ny, nz))
    return nothing
end

"""
    weno5_advect!(Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant, precision)

`ht3d_weno5_advect` (include/ht3d.h).
"""
function weno5_advect!(Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant, precision; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _check(ctx, C.ht3d_weno5_advect(ctx.ptr, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, Cint[bc_type6...], Cdouble[bc_val6...], variant, precision, nx, ny, nz))
    return nothing
end

"""
    weno5_advect_f32!(Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant)

`ht3d_weno5_advect_f32` (include/ht3d.h).
"""
function weno5_advect_f32!(Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _check(ctx, C.ht3d_weno5_advect_f32(ctx.ptr, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, Cint[bc_type6...], Cdouble[bc_val6...], variant, nx, ny, nz))
    return nothing
end

"""
    step_hrl!(Tc_ex, Pc_ex, ktv, kfv, Vx, Vy, Vz, p, precision)

`ht3d_step_hrl` (include/ht3d.h); returns st_thermal, st_darcy.
"""
function step_hrl!(Tc_ex, Pc_ex, ktv, kfv, Vx, Vy, Vz, p, precision; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    st_thermal = Ref{DyrelStats}()
    st_darcy = Ref{DyrelStats}()
    _check(ctx, C.ht3d_step_hrl(ctx.ptr, Tc_ex, Pc_ex, ktv, kfv, Vx, Vy, Vz, p, st_thermal, st_darcy, precision, nx, ny, nz))
    return st_thermal[], st_darcy[]
end

"""
    step_v18!(Tc_ex, Pc_ex, phc_ex, phv, wN, kmul_v, Vx, Vy, Vz, p)

`ht3d_step_v18` (include/ht3d.h); returns st_thermal, st_darcy.
"""
function step_v18!(Tc_ex, Pc_ex, phc_ex, phv, wN, kmul_v, Vx, Vy, Vz, p; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    st_thermal = Ref{DyrelStats}()
    st_darcy = Ref{DyrelStats}()
    _check(ctx, C.ht3d_step_v18(ctx.ptr, Tc_ex, Pc_ex, phc_ex, phv, wN, kmul_v, Vx, Vy, Vz, p, st_thermal, st_darcy, nx, ny, nz))
    return st_thermal[], st_darcy[]
end

"""
    postprocess_fields!(out, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, prm)

`ht3d_postprocess_fields` (include/ht3d.h).
"""
function postprocess_fields!(out, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, prm; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _check(ctx, C.ht3d_postprocess_fields(ctx.ptr, out, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, prm, nx, ny, nz))
    return nothing
end

"""
    SetInitialConditions_Khaled!(phc_ex, phv, wN, geom, Tc_ex, Pc_ex, Tbot, Ttop, Pbot, Ptop, xmin, ymin, zmin, xmax, ymax, zmax, L)

`ht3d_SetInitialConditions_Khaled` (include/ht3d.h).
"""
function SetInitialConditions_Khaled!(phc_ex, phv, wN, geom, Tc_ex, Pc_ex, Tbot, Ttop, Pbot, Ptop, xmin, ymin, zmin, xmax, ymax, zmax, L; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _check(ctx, C.ht3d_SetInitialConditions_Khaled(ctx.ptr, phc_ex, phv, wN, geom, Tc_ex, Pc_ex, Tbot, Ttop, Pbot, Ptop, xmin, ymin, zmin, xmax, ymax, zmax, L, nx, ny, nz))
    return nothing
end

"""
    Nusselt(qy, Lx, Lz)

`ht3d_Nusselt` (include/ht3d.h); returns Nu.
"""
function Nusselt(qy, Lx, Lz; ctx::Context = context())
    nx, ny, nz = size(qy) .- (0, 1, 0)
    Nu = Ref{Cdouble}()
    _check(ctx, C.ht3d_Nusselt(ctx.ptr, qy, Lx, Lz, nx, ny, nz, Nu))
    return Nu[]
end

"""
    breakpoint_write(path, Tc_ex, Pc_ex, time, dt)

`ht3d_breakpoint_write` (include/ht3d.h).
"""
function breakpoint_write(path, Tc_ex, Pc_ex, time, dt; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _check(ctx, C.ht3d_breakpoint_write(ctx.ptr, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz))
    return nothing
end

"""
    breakpoint_read!(path, Tc_ex, Pc_ex)

`ht3d_breakpoint_read` (include/ht3d.h); returns time, dt.
"""
function breakpoint_read!(path, Tc_ex, Pc_ex; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    time = Ref{Cdouble}()
    dt = Ref{Cdouble}()
    _check(ctx, C.ht3d_breakpoint_read(ctx.ptr, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz))
    return time[], dt[]
end

"""
    breakpoint_write_h5(path, Tc_ex, Pc_ex, time, dt)

`ht3d_breakpoint_write_h5` (include/ht3d.h).
"""
function breakpoint_write_h5(path, Tc_ex, Pc_ex, time, dt; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    _check(ctx, C.ht3d_breakpoint_write_h5(ctx.ptr, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz))
    return nothing
end

"""
    breakpoint_read_h5!(path, Tc_ex, Pc_ex)

`ht3d_breakpoint_read_h5` (include/ht3d.h); returns time, dt.
"""
function breakpoint_read_h5!(path, Tc_ex, Pc_ex; ctx::Context = context())
    nx, ny, nz = size(Tc_ex) .- 2
    time = Ref{Cdouble}()
    dt = Ref{Cdouble}()
    _check(ctx, C.ht3d_breakpoint_read_h5(ctx.ptr, path, Tc_ex, Pc_ex, time, dt, nx, ny, nz))
    return time[], dt[]
end

"""
    ensemble_step!(members::Vector{Instance}, precision)

One time step of every member (`ht3d_ensemble_step`); returns the members' statuses.
"""
function ensemble_step!(members::Vector{Instance}, precision; ctx::Context = context())
    st = GC.@preserve members C.ht3d_ensemble_step(ctx.ptr, pointer(members), Cint(length(members)), Cint(precision))
    st == OK || st == ERR_NAN || st == ERR_DIVERGED || _check(ctx, st)
    return [m.status for m in members]
end

end  # module HT3D
