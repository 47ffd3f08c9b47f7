// WENO5 advection with FP32 storage and arithmetic: the same SSP-RK2
// dimension-split sweep as ht3d_weno5_advect (tools/Weno5_Routines.jl /
// tools/Weno5_Routines_v2.jl) on float fields, for the standalone sweep of
// the large-grid workload.  The epsilon floor of the weights is 1e-18 instead
// of 1e-99 (see weno5_f32).
#include "weno_core.cuh"

namespace {

template <int AXIS, int QUIRK, int STAGE>
__global__ void __launch_bounds__(256) k_weno_stage_f32(const float* __restrict__ src, float* dst, const float* T0,
                                                        const float* __restrict__ V, float dt, float h, WenoBC bc,
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
    const float* line = src + e - (long long)idx * stride;
    float x[7];
#pragma unroll
    for (int o = 0; o < 7; ++o) x[o] = line_at<float>(line, stride, idx + o - 3, n, bc);
    long long vl, vs;
    if (AXIS == 0) { vl = ix3(i, j, k, nx + 1, ny); vs = 1; }
    else if (AXIS == 1) { vl = ix3(i, j, k, nx, ny + 1); vs = nx; }
    else { vl = ix3(i, j, k, nx, ny); vs = (long long)nx * ny; }
    const float a = V[vl], b = V[vl + vs];
    const float Vm = a < 0.0f ? a : 0.0f;
    const float Vp = b >= 0.0f ? b : 0.0f;
    float d[6];
#pragma unroll
    for (int o = 0; o < 6; ++o) d[o] = h * (x[o + 1] - x[o]);
    const float m5 = QUIRK ? h * (x[5] - x[2]) : d[4];
    const float dFm = weno5_f32(d[0], d[1], d[2], d[3], m5);
    const float dFp = weno5_f32(d[5], d[4], d[3], d[2], d[1]);
    const float t = x[3] - dt * (Vp * dFm + Vm * dFp);
    if (STAGE == 1) dst[e] = t;
    else dst[e] = 0.5f * t + 0.5f * T0[e];
}

template <int AXIS, int QUIRK>
void axis_f32(ht3d_ctx* ctx, float* T, float* T1, const float* V, float dt, float h, WenoBC bc, int nx, int ny, int nz) {
    dim3 b(32, 8, 1), g((nx + 31) / 32, (ny + 7) / 8, nz);
    HT3D_LAUNCH(ctx, (k_weno_stage_f32<AXIS, QUIRK, 1>), g, b, 0, T, T1, (const float*)nullptr, V, dt, h, bc, nx, ny, nz);
    HT3D_LAUNCH(ctx, (k_weno_stage_f32<AXIS, QUIRK, 2>), g, b, 0, T1, T, T, V, dt, h, bc, nx, ny, nz);
}

template <int QUIRK>
void all_f32(ht3d_ctx* ctx, float* T, float* T1, const float* const* V, float dt, const float* h, const WenoBC* bc,
             int nx, int ny, int nz) {
    axis_f32<0, QUIRK>(ctx, T, T1, V[0], dt, h[0], bc[0], nx, ny, nz);
    axis_f32<1, QUIRK>(ctx, T, T1, V[1], dt, h[1], bc[1], nx, ny, nz);
    axis_f32<2, QUIRK>(ctx, T, T1, V[2], dt, h[2], bc[2], nx, ny, nz);
}

}  // namespace

extern "C" int ht3d_weno5_advect_f32(ht3d_ctx* ctx, float* Tc_ex, const float* Vx, const float* Vy, const float* Vz,
                                     double dt, double _dx, double _dy, double _dz, const int* bc_type6,
                                     const double* bc_val6, int variant, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        ht3d_check_dims(nx, ny, nz, 3);
        HT3D_REQUIRE(Tc_ex && Vx && Vy && Vz && bc_type6 && bc_val6, "null argument");
        HT3D_REQUIRE(variant >= HT3D_WENO_V1 && variant <= HT3D_WENO_V2_FIXED, "unknown WENO variant");
        WenoBC bc[3];
        for (int a = 0; a < 3; ++a) {
            HT3D_REQUIRE(bc_type6[2 * a] >= 0 && bc_type6[2 * a] <= 2 && bc_type6[2 * a + 1] >= 0 &&
                         bc_type6[2 * a + 1] <= 2, "WENO BC type must be 0, 1 or 2");
            bc[a] = WenoBC{bc_type6[2 * a], bc_type6[2 * a + 1], bc_val6[2 * a], bc_val6[2 * a + 1]};
        }
        const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
        float* T1 = (float*)ht3d_scratch(ctx, SLOT_AUX3, sizeof(float) * nex);
        const float* V[3] = {Vx, Vy, Vz};
        const float h[3] = {(float)_dx, (float)_dy, (float)_dz};
        if (variant == HT3D_WENO_V2_REF) all_f32<1>(ctx, Tc_ex, T1, V, (float)dt, h, bc, nx, ny, nz);
        else all_f32<0>(ctx, Tc_ex, T1, V, (float)dt, h, bc, nx, ny, nz);
        return HT3D_OK;
    });
}
