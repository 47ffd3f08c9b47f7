// WENO5 temperature advection (tools/Weno5_Routines.jl, tools/Weno5_Routines_v2.jl).
//
// Two layers:
//  * granular drop-ins that mirror the reference kernels one for one
//    (VxPlusMinus!, Gradients_*_Weno5!, dFdx_Weno5!, Boundaries_*_Weno5!,
//    Advect!, TimeAveraging!), and
//  * the fused sweep used by the solver: per axis two launches (the two
//    SSP-RK2 stages), ghost values evaluated on the fly from the boundary
//    rules (no (n+6)^3 buffer, no v1..v5 temporaries), the RK averaging fused
//    into the second stage.
#include "ht3d_internal.cuh"
#include "weno_core.cuh"

namespace {

// One SSP-RK2 stage along AXIS on ghosted (ex) fields.
//   PREC 0: FP64 reference-order arithmetic (parity form; this translation
//           unit is compiled with -fmad=false)
//   PREC 1: mixed form: FP64 state, differences, central candidate and
//           corrections; FP32 smoothness indicators and weights (weno5_mixed)
//   STAGE 1: dst = src - dt*(Vp*dFm + Vm*dFp)
//   STAGE 2: dst = 0.5*(src - dt*(...)) + 0.5*T0   (TimeAveraging!, order 2)
template <int AXIS, int QUIRK, int STAGE, int PREC>
__global__ void __launch_bounds__(256) k_weno_stage(const double* __restrict__ src, double* dst, const double* T0,
                                                    const double* __restrict__ V, double dt, double h, WenoBC bc,
                                                    int nx, int ny, int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= nx || j >= ny || k >= nz) return;
    const int n1 = nx + 2, n2 = ny + 2;
    const long long e = (i + 1) + (long long)n1 * ((j + 1) + (long long)n2 * (k + 1));
    const int idx = AXIS == 0 ? i : (AXIS == 1 ? j : k);
    const int n = AXIS == 0 ? nx : (AXIS == 1 ? ny : nz);
    const long long stride = AXIS == 0 ? 1 : (AXIS == 1 ? (long long)n1 : (long long)n1 * n2);
    const double* line = src + e - (long long)idx * stride;
    double x[7];
#pragma unroll
    for (int o = 0; o < 7; ++o) x[o] = line_at(line, stride, idx + o - 3, n, bc);
    // face velocities: V[idx] (left) and V[idx+1] (right) along AXIS
    long long vl;
    long long vs;
    if (AXIS == 0) { vl = ix3(i, j, k, nx + 1, ny); vs = 1; }
    else if (AXIS == 1) { vl = ix3(i, j, k, nx, ny + 1); vs = nx; }
    else { vl = ix3(i, j, k, nx, ny); vs = (long long)nx * ny; }
    const double a = V[vl], b = V[vl + vs];
    const double Vm = a < 0.0 ? a : 0.0;
    const double Vp = b >= 0.0 ? b : 0.0;
    double rhs;
    if (PREC == 0) {
        // x[o] holds X[I+o-3]
        const double m1 = h * (x[1] - x[0]), m2 = h * (x[2] - x[1]), m3 = h * (x[3] - x[2]), m4 = h * (x[4] - x[3]);
        const double m5 = QUIRK ? h * (x[5] - x[2]) : h * (x[5] - x[4]);
        const double dFm = upwind_active(Vp) ? weno5_ref(m1, m2, m3, m4, m5) : 0.0;
        const double p1 = h * (x[6] - x[5]), p2 = h * (x[5] - x[4]), p3 = h * (x[4] - x[3]), p4 = h * (x[3] - x[2]);
        const double p5 = h * (x[2] - x[1]);
        const double dFp = upwind_active(Vm) ? weno5_ref(p1, p2, p3, p4, p5) : 0.0;
        rhs = Vp * dFm + Vm * dFp;
    } else {
        // FP64 differences e[o] = X[I+o-2] - X[I+o-3]; FP32 copies scaled by h
        // for the smoothness indicators (weno5_mixed)
        double e[6];
        float f[6];
        const float hf = (float)h;
#pragma unroll
        for (int o = 0; o < 6; ++o) {
            e[o] = x[o + 1] - x[o];
            f[o] = hf * (float)e[o];
        }
        const double e5 = QUIRK ? x[5] - x[2] : e[4];
        const float f5 = QUIRK ? hf * (float)e5 : f[4];
        const double dFm = upwind_active(Vp) ? h * weno5_mixed(e[0], e[1], e[2], e[3], e5, f[0], f[1], f[2], f[3], f5)
                                             : 0.0;
        const double dFp = upwind_active(Vm) ? h * weno5_mixed(e[5], e[4], e[3], e[2], e[1], f[5], f[4], f[3], f[2], f[1])
                                             : 0.0;
        rhs = Vp * dFm + Vm * dFp;
    }
    const double t = x[3] - dt * rhs;
    if (STAGE == 1) dst[e] = t;
    else dst[e] = 0.5 * t + 0.5 * T0[e];
}

// ------------------------------------------------------- granular drop-ins
#define GIDX                                             \
    const int i = blockIdx.x * blockDim.x + threadIdx.x; \
    const int j = blockIdx.y * blockDim.y + threadIdx.y; \
    const int k = blockIdx.z * blockDim.z + threadIdx.z

// a zero (or NaN) face velocity leaves the output as it was, as in the reference
__global__ void k_vplusminus(double* Vm, double* Vp, const double* __restrict__ V, int axis, int nx, int ny, int nz) {
    for_cells_z(nx, ny, nz, [&](int i, int j, int k) {
        const int c = ix3(i, j, k, nx, ny);
        const int v1 =
            axis == 0 ? ix3(i, j, k, nx + 1, ny) : (axis == 1 ? ix3(i, j, k, nx, ny + 1) : ix3(i, j, k, nx, ny));
        const int v2 = axis == 0 ? v1 + 1 : (axis == 1 ? v1 + nx : v1 + nx * ny);
        const double a = V[v1], b = V[v2];
        const int sa = cmp_sign(a), sb = cmp_sign(b);
        if (sa < 0) Vm[c] = a;
        if (sa > 0) Vm[c] = 0.0;
        if (sb < 0) Vp[c] = 0.0;
        if (sb > 0) Vp[c] = b;
    });
}

__global__ void k_dfdx(double* dF, const double* __restrict__ v1, const double* __restrict__ v2,
                       const double* __restrict__ v3, const double* __restrict__ v4, const double* __restrict__ v5,
                       long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dF[t] = weno5_ref(v1[t], v2[t], v3[t], v4[t], v5[t]);
}

__global__ void k_gradients(double* v1, double* v2, double* v3, double* v4, double* v5, const double* __restrict__ X,
                            int axis, int sign, double h, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const int n1 = nx + 6, n2 = ny + 6;
    const long long base = ix3(i + 3, j + 3, k + 3, n1, n2);
    const long long st = axis == 0 ? 1 : (axis == 1 ? n1 : (long long)n1 * n2);
    auto x = [&](int o) { return X[base + o * st]; };
    const int c = ix3(i, j, k, nx, ny);
    if (sign < 0) {
        v1[c] = h * (x(-2) - x(-3));
        v2[c] = h * (x(-1) - x(-2));
        v3[c] = h * (x(0) - x(-1));
        v4[c] = h * (x(1) - x(0));
        v5[c] = h * (x(2) - x(1));
    } else {
        v1[c] = h * (x(3) - x(2));
        v2[c] = h * (x(2) - x(1));
        v3[c] = h * (x(1) - x(0));
        v4[c] = h * (x(0) - x(-1));
        v5[c] = h * (x(-1) - x(-2));
    }
}

__global__ void k_boundaries(double* X, const double* __restrict__ Fc, int axis, WenoBC bc, int o, int nx, int ny,
                             int nz) {
    GIDX;
    const int n1 = nx + 6, n2 = ny + 6, n3 = nz + 6;
    if (i >= n1 || j >= n2 || k >= n3) return;
    const int f1 = nx + 2 * o, f2 = ny + 2 * o;
    if (i < nx && j < ny && k < nz) X[ix3(i + 3, j + 3, k + 3, n1, n2)] = Fc[ix3(i + o, j + o, k + o, f1, f2)];
    const int idx[3] = {i, j, k};
    const int N[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a)
        if (a != axis && !(idx[a] >= 3 && idx[a] < N[a] + 3)) return;
    const int p = idx[axis], n = N[axis];
    int s[3] = {i - 3, j - 3, k - 3};
    if (p < 3) {
        if (bc.typeL == HT3D_BC_PERIODIC) s[axis] = n - 3 + p;
        else s[axis] = 2 - p;
        const double v = Fc[ix3(s[0] + o, s[1] + o, s[2] + o, f1, f2)];
        X[ix3(i, j, k, n1, n2)] = bc.typeL == HT3D_BC_DIRICHLET ? 2 * bc.valL - v : v;
    } else if (p >= n + 3) {
        const int q = p - (n + 3);
        if (bc.typeR == HT3D_BC_PERIODIC) s[axis] = q;
        else s[axis] = n - 1 - q;
        const double v = Fc[ix3(s[0] + o, s[1] + o, s[2] + o, f1, f2)];
        X[ix3(i, j, k, n1, n2)] = bc.typeR == HT3D_BC_DIRICHLET ? 2 * bc.valR - v : v;
    }
}

__global__ void k_advect_v1(double* Fc, const double* __restrict__ Vxp, const double* __restrict__ dm,
                            const double* __restrict__ Vxm, const double* __restrict__ dp, double dt, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        Fc[t] = Fc[t] - dt * (Vxp[t] * dm[t] + Vxm[t] * dp[t]);
}
// TimeAveraging!: Fc = (1/order) Fc + (1 - 1/order) Fold.  The two weights
// a = 1/order and b = 1 - a are formed once on the host (IEEE division and
// subtraction, the same bits as per cell) and passed in.
__global__ void k_timeavg_v1(double* Fc, const double* __restrict__ Fold, double a, double b, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        Fc[t] = a * Fc[t] + b * Fold[t];
}
__global__ void k_timeavg_v2(double* Fc, const double* __restrict__ Fold, double a, double b, int nx, int ny, int nz) {
    for_cells_z(nx, ny, nz, [&](int i, int j, int k) {
        const long long e = ix3(i + 1, j + 1, k + 1, nx + 2, ny + 2);
        Fc[e] = a * Fc[e] + b * Fold[ix3(i, j, k, nx, ny)];
    });
}

// Advect! v2 (tools/Weno5_Routines_v2.jl:55-212), reference arithmetic
__global__ void k_advect_v2(double* Fc, const double* __restrict__ X, const double* __restrict__ V, int axis, double dt,
                            double h, int quirk, int nx, int ny, int nz) {
    GIDX;
    if (i >= nx || j >= ny || k >= nz) return;
    const int n1 = nx + 6, n2 = ny + 6;
    const long long base = ix3(i + 3, j + 3, k + 3, n1, n2);
    const long long st = axis == 0 ? 1 : (axis == 1 ? n1 : (long long)n1 * n2);
    auto x = [&](int o) { return X[base + o * st]; };
    const int v1 = axis == 0 ? ix3(i, j, k, nx + 1, ny) : (axis == 1 ? ix3(i, j, k, nx, ny + 1) : ix3(i, j, k, nx, ny));
    const int v2 = axis == 0 ? v1 + 1 : (axis == 1 ? v1 + nx : v1 + nx * ny);
    const double a = V[v1], b = V[v2];
    double Vm = 0.0, Vp = 0.0;
    if (a < 0.0) Vm = a;
    if (a >= 0.0) Vm = 0.0;
    if (b < 0.0) Vp = 0.0;
    if (b >= 0.0) Vp = b;
    // both derivatives always, as the reference kernel: on a field whose
    // velocity sign changes from face to face, skipping a zero-factor
    // derivative (as the fused stages do) made this kernel 13 % slower
    const double dFm = weno5_ref(h * (x(-2) - x(-3)), h * (x(-1) - x(-2)), h * (x(0) - x(-1)), h * (x(1) - x(0)),
                                 quirk ? h * (x(2) - x(-1)) : h * (x(2) - x(1)));
    const double dFp = weno5_ref(h * (x(3) - x(2)), h * (x(2) - x(1)), h * (x(1) - x(0)), h * (x(0) - x(-1)),
                                 h * (x(-1) - x(-2)));
    const long long e = ix3(i + 1, j + 1, k + 1, nx + 2, ny + 2);
    Fc[e] = Fc[e] - dt * (Vp * dFm + Vm * dFp);
}

inline dim3 g1(ht3d_ctx* ctx, long long n) {
    long long b = (n + 255) / 256;
    return dim3((unsigned)std::max<long long>(1, std::min<long long>(b, (long long)ctx->num_sms * 16)));
}

template <int AXIS, int QUIRK, int PREC>
void weno_axis(ht3d_ctx* ctx, double* T, double* T1, const double* V, double dt, double h, WenoBC bc, int nx, int ny,
               int nz) {
    dim3 b(32, 8, 1), g((nx + 31) / 32, (ny + 7) / 8, nz);
    HT3D_LAUNCH(ctx, (k_weno_stage<AXIS, QUIRK, 1, PREC>), g, b, 0, T, T1, (const double*)nullptr, V, dt, h, bc, nx,
                ny, nz);
    HT3D_LAUNCH(ctx, (k_weno_stage<AXIS, QUIRK, 2, PREC>), g, b, 0, T1, T, T, V, dt, h, bc, nx, ny, nz);
}

template <int QUIRK, int PREC>
void weno_all(ht3d_ctx* ctx, double* T, double* T1, const double* const* V, double dt, const double* h,
              const WenoBC* bc, int nx, int ny, int nz) {
    weno_axis<0, QUIRK, PREC>(ctx, T, T1, V[0], dt, h[0], bc[0], nx, ny, nz);
    weno_axis<1, QUIRK, PREC>(ctx, T, T1, V[1], dt, h[1], bc[1], nx, ny, nz);
    weno_axis<2, QUIRK, PREC>(ctx, T, T1, V[2], dt, h[2], bc[2], nx, ny, nz);
}

}  // namespace

// used by the step driver
void ht3d_weno5_advect_impl(ht3d_ctx* ctx, double* Tc_ex, const double* Vx, const double* Vy, const double* Vz,
                            double dt, double _dx, double _dy, double _dz, const int* bc_type6, const double* bc_val6,
                            int variant, int precision, int nx, int ny, int nz) {
    NvtxRange range("ht3d WENO5 advection");
    ht3d_check_dims(nx, ny, nz, 3);
    HT3D_REQUIRE(variant >= HT3D_WENO_V1 && variant <= HT3D_WENO_V2_FIXED, "unknown WENO variant");
    HT3D_REQUIRE(precision == HT3D_FP64 || precision == HT3D_MIXED, "unknown precision");
    WenoBC bc[3];
    for (int a = 0; a < 3; ++a) {
        HT3D_REQUIRE(bc_type6[2 * a] >= 0 && bc_type6[2 * a] <= 2 && bc_type6[2 * a + 1] >= 0 && bc_type6[2 * a + 1] <= 2,
                     "WENO BC type must be 0, 1 or 2");
        bc[a].typeL = bc_type6[2 * a];
        bc[a].typeR = bc_type6[2 * a + 1];
        bc[a].valL = bc_val6[2 * a];
        bc[a].valR = bc_val6[2 * a + 1];
    }
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    double* T1 = (double*)ht3d_scratch(ctx, SLOT_WENO_T1, sizeof(double) * nex);
    const double* V[3] = {Vx, Vy, Vz};
    const double h[3] = {_dx, _dy, _dz};
    const bool quirk = variant == HT3D_WENO_V2_REF;
    if (precision == HT3D_FP64) {
        if (quirk) weno_all<1, 0>(ctx, Tc_ex, T1, V, dt, h, bc, nx, ny, nz);
        else weno_all<0, 0>(ctx, Tc_ex, T1, V, dt, h, bc, nx, ny, nz);
    } else {
        bool periodic = false;
        for (int a = 0; a < 3; ++a)
            periodic = periodic || bc[a].typeL == HT3D_BC_PERIODIC || bc[a].typeR == HT3D_BC_PERIODIC;
        if (!periodic) ht3d_weno5_mixed_march(ctx, Tc_ex, T1, V, dt, h, bc_type6, bc_val6, quirk, nx, ny, nz);
        else if (quirk) weno_all<1, 1>(ctx, Tc_ex, T1, V, dt, h, bc, nx, ny, nz);
        else weno_all<0, 1>(ctx, Tc_ex, T1, V, dt, h, bc, nx, ny, nz);
    }
}

extern "C" {

#define G3(a, b, c) grid3((a), (b), (c), kBlock3)

int ht3d_VPlusMinus(ht3d_ctx* ctx, double* Vm, double* Vp, const double* V, int axis, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Vm, Vp, V), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        HT3D_REQUIRE(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
        HT3D_LAUNCH(ctx, k_vplusminus, grid3z(nx, ny, nz), kBlock3, 0, Vm, Vp, V, axis, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_dFdx_Weno5(ht3d_ctx* ctx, double* dFdxi, const double* V1, const double* V2, const double* V3,
                    const double* V4, const double* V5, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(dFdxi, V1, V2, V3, V4, V5), "null argument");
        HT3D_REQUIRE(n >= 0, "negative size");
        if (n) HT3D_LAUNCH(ctx, k_dfdx, g1(ctx, n), 256, 0, dFdxi, V1, V2, V3, V4, V5, n);
        return HT3D_OK;
    });
}

int ht3d_Gradients_Weno5(ht3d_ctx* ctx, double* v1, double* v2, double* v3, double* v4, double* v5,
                         const double* Fc_exxx, int axis, int sign, double _dx, double _dy, double _dz, int nx, int ny,
                         int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(v1, v2, v3, v4, v5, Fc_exxx), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        HT3D_REQUIRE(axis >= 0 && axis <= 2 && (sign == 1 || sign == -1), "bad axis/sign");
        const double h = axis == 0 ? _dx : (axis == 1 ? _dy : _dz);
        HT3D_LAUNCH(ctx, k_gradients, G3(nx, ny, nz), kBlock3, 0, v1, v2, v3, v4, v5, Fc_exxx, axis, sign, h, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_Boundaries_Weno5(ht3d_ctx* ctx, double* Fc_exxx, const double* Fc, int axis, int type_L, double val_L,
                          int type_R, double val_R, int fc_ghosted, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Fc_exxx, Fc), "null argument");
        ht3d_check_dims(nx, ny, nz, 3);
        HT3D_REQUIRE(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
        HT3D_REQUIRE(type_L >= 0 && type_L <= 2 && type_R >= 0 && type_R <= 2, "BC type must be 0, 1 or 2");
        WenoBC bc{type_L, type_R, val_L, val_R};
        HT3D_LAUNCH(ctx, k_boundaries, G3(nx + 6, ny + 6, nz + 6), kBlock3, 0, Fc_exxx, Fc, axis, bc, fc_ghosted ? 1 : 0,
                    nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_Advect_v1(ht3d_ctx* ctx, double* Fc, const double* Vxp, const double* dTdxm, const double* Vxm,
                   const double* dTdxp, double dt, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Fc, Vxp, dTdxm, Vxm, dTdxp), "null argument");
        HT3D_REQUIRE(n >= 0, "negative size");
        if (n) HT3D_LAUNCH(ctx, k_advect_v1, g1(ctx, n), 256, 0, Fc, Vxp, dTdxm, Vxm, dTdxp, dt, n);
        return HT3D_OK;
    });
}

int ht3d_TimeAveraging_v1(ht3d_ctx* ctx, double* Fc, const double* Fold, double order, long long n) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Fc, Fold), "null argument");
        HT3D_REQUIRE(n >= 0, "negative size");
        const double a = 1.0 / order, b = 1.0 - a;
        if (n) HT3D_LAUNCH(ctx, k_timeavg_v1, g1(ctx, n), 256, 0, Fc, Fold, a, b, n);
        return HT3D_OK;
    });
}

int ht3d_Advect_v2(ht3d_ctx* ctx, double* Fc_ex, const double* X_exxx, const double* V, int axis, double dt,
                   double _dx, double _dy, double _dz, int quirk, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Fc_ex, X_exxx, V), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        HT3D_REQUIRE(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
        const double h = axis == 0 ? _dx : (axis == 1 ? _dy : _dz);
        HT3D_LAUNCH(ctx, k_advect_v2, G3(nx, ny, nz), kBlock3, 0, Fc_ex, X_exxx, V, axis, dt, h, quirk ? 1 : 0, nx, ny,
                    nz);
        return HT3D_OK;
    });
}

int ht3d_TimeAveraging_v2(ht3d_ctx* ctx, double* Fc_ex, const double* Fold, double order, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Fc_ex, Fold), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        const double a = 1.0 / order, b = 1.0 - a;
        HT3D_LAUNCH(ctx, k_timeavg_v2, grid3z(nx, ny, nz), kBlock3, 0, Fc_ex, Fold, a, b, nx, ny, nz);
        return HT3D_OK;
    });
}

int ht3d_weno5_advect(ht3d_ctx* ctx, double* Tc_ex, const double* Vx, const double* Vy, const double* Vz, double dt,
                      double _dx, double _dy, double _dz, const int* bc_type6, const double* bc_val6, int variant,
                      int precision, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(Tc_ex && Vx && Vy && Vz && bc_type6 && bc_val6, "null argument");
        ht3d_weno5_advect_impl(ctx, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant, precision, nx, ny,
                               nz);
        return HT3D_OK;
    });
}

}  // extern "C"
