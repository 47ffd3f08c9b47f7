// WENO5 advection with FP32 storage and arithmetic: the same SSP-RK2
// dimension-split sweep as ht3d_weno5_advect (tools/Weno5_Routines.jl /
// tools/Weno5_Routines_v2.jl) on float fields, for the standalone sweep of
// the large-grid workload.  The epsilon floor of the weights is 1e-18 instead
// of 1e-99 (see weno5_f32).  Both stages of an axis run in one kernel (rows in
// shared memory along x, register windows marching along y and z), so every
// axis reads T and V once and writes T once; periodic y/z axes use one launch
// per stage.
#include "weno_core.cuh"

namespace {

// One point of one SSP-RK2 stage from its 7-point window x0..x6 along the
// sweep axis (the Advect! update of tools/Weno5_Routines_v2.jl:55-212):
// upwind WENO5 derivatives from both sides, weighted by the face velocities
// a (left face) and b (right face).
template <int QUIRK>
__device__ __forceinline__ float weno_point_f32(float x0, float x1, float x2, float x3, float x4, float x5, float x6,
                                                float a, float b, float dt, float h) {
    const float Vm = a < 0.0f ? a : 0.0f;
    const float Vp = b >= 0.0f ? b : 0.0f;
    const float d0 = h * (x1 - x0), d1 = h * (x2 - x1), d2 = h * (x3 - x2), d3 = h * (x4 - x3), d4 = h * (x5 - x4),
                d5 = h * (x6 - x5);
    const float m5 = QUIRK ? h * (x5 - x2) : d4;
    const float dFm = upwind_active(Vp) ? weno5_f32(d0, d1, d2, d3, m5) : 0.0f;
    const float dFp = upwind_active(Vm) ? weno5_f32(d5, d4, d3, d2, d1) : 0.0f;
    return x3 - dt * (Vp * dFm + Vm * dFp);
}

// The same point from its six one-sided differences d[o] = h (x[o+1] - x[o])
// (the march kernels keep them in a window: one new difference per point);
// x2, x5 only for the v2 stencil quirk, x3 the point itself.
template <int QUIRK>
__device__ __forceinline__ float weno_point_f32_d(const float (&d)[6], float x2, float x3, float x5, float a, float b,
                                                  float dt, float h) {
    const float Vm = a < 0.0f ? a : 0.0f;
    const float Vp = b >= 0.0f ? b : 0.0f;
    const float m5 = QUIRK ? h * (x5 - x2) : d[4];
    const float dFm = upwind_active(Vp) ? weno5_f32(d[0], d[1], d[2], d[3], m5) : 0.0f;
    const float dFp = upwind_active(Vm) ? weno5_f32(d[5], d[4], d[3], d[2], d[1]) : 0.0f;
    return x3 - dt * (Vp * dFm + Vm * dFp);
}

// ghost value at position p (< 0 or >= n) from its mirror value v
__device__ __forceinline__ float weno_ghost(float v, bool left, const WenoBC& bc) {
    const int t = left ? bc.typeL : bc.typeR;
    return t == HT3D_BC_DIRICHLET ? (float)(2 * (left ? bc.valL : bc.valR)) - v : v;
}

// Unfused stage (any BC, incl. periodic): one launch per stage and axis.
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
    const float t = weno_point_f32<QUIRK>(x[0], x[1], x[2], x[3], x[4], x[5], x[6], V[vl], V[vl + vs], dt, h);
    if (STAGE == 1) dst[e] = t;
    else dst[e] = 0.5f * t + 0.5f * T0[e];
}

// Both stages of one axis fused, x-axis: a warp owns a row; the row of T0 and
// of the stage-1 result T1 live in shared memory with three ghost cells on
// each side (filled by the BC rules after each stage), so the stencils are
// plain shared loads.  Reads T0 and Vx once and writes T once.
constexpr int kRowWarps = 8;

// ghost cells r[-3..-1] and r[n..n+2] of a shared row r (r points at element 0)
__device__ __forceinline__ void fill_row_ghosts(float* r, int n, const WenoBC& bc, int lane) {
    if (lane < 3) {  // left: position -1-q mirrors q (periodic: n-1-q)
        const int q = lane;
        r[-1 - q] = bc.typeL == HT3D_BC_PERIODIC ? r[n - 1 - q] : weno_ghost(r[q], true, bc);
    } else if (lane < 6) {  // right: position n+q mirrors n-1-q (periodic: q)
        const int q = lane - 3;
        r[n + q] = bc.typeR == HT3D_BC_PERIODIC ? r[q] : weno_ghost(r[n - 1 - q], false, bc);
    }
}

template <int QUIRK>
__global__ void __launch_bounds__(32 * kRowWarps) k_weno_rows_f32(float* __restrict__ T, const float* __restrict__ Vx,
                                                                  float dt, float h, WenoBC bc, int nx, int ny,
                                                                  int nz) {
    extern __shared__ float rows_sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long row = (long long)blockIdx.x * kRowWarps + warp;  // over (j, k)
    if (row >= (long long)ny * nz) return;                           // whole warps only
    const int j = (int)(row % ny), k = (int)(row / ny);
    float* s0 = rows_sm + (size_t)warp * 2 * (nx + 6) + 3;  // T0[-3 .. nx+2]
    float* s1 = s0 + nx + 6;                                 // T1[-3 .. nx+2]
    float* line = T + 1 + (long long)(nx + 2) * ((j + 1) + (long long)(ny + 2) * (k + 1));
    const float* vrow = Vx + (long long)(nx + 1) * (j + (long long)ny * k);
    for (int m = lane; m < nx; m += 32) s0[m] = line[m];
    __syncwarp();
    fill_row_ghosts(s0, nx, bc, lane);
    __syncwarp();
    for (int m = lane; m < nx; m += 32) {
        const float* x = s0 + m - 3;
        s1[m] = weno_point_f32<QUIRK>(x[0], x[1], x[2], x[3], x[4], x[5], x[6], vrow[m], vrow[m + 1], dt, h);
    }
    __syncwarp();
    fill_row_ghosts(s1, nx, bc, lane);
    __syncwarp();
    for (int m = lane; m < nx; m += 32) {
        const float* x = s1 + m - 3;
        const float t = weno_point_f32<QUIRK>(x[0], x[1], x[2], x[3], x[4], x[5], x[6], vrow[m], vrow[m + 1], dt, h);
        line[m] = 0.5f * t + 0.5f * s0[m];
    }
}

// Both stages of one axis fused, y or z axis (Neumann / Dirichlet ends),
// out of place (src -> dst, the inner cells): a thread marches along a chunk
// [c0, c0 + L) of its line with sliding register windows
//   w0 = T0[c .. c+6], w1 = T1[c-3 .. c+3], v = V faces c .. c+4,
// producing T1[c+3] and then T[c]; the first six T1 values of a chunk (and
// the ghosts at the line's ends) are produced before the march.  Threads are
// consecutive in x (coalesced); chunks multiply the parallelism of the lines.
constexpr int kMarchL = 64;

template <int AXIS, int QUIRK>
__global__ void __launch_bounds__(128) k_weno_march_f32(const float* __restrict__ src, float* __restrict__ dst,
                                                        const float* __restrict__ V, float dt, float h, WenoBC bc,
                                                        int nx, int ny, int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int o = blockIdx.y;  // k for the y-march, j for the z-march
    const int c0 = blockIdx.z * kMarchL;
    const int n = AXIS == 1 ? ny : nz;
    if (i >= nx || c0 >= n) return;
    const int c1 = min(n, c0 + kMarchL);
    const int n1 = nx + 2, n2 = ny + 2;
    const long long stride = AXIS == 1 ? (long long)n1 : (long long)n1 * n2;
    const long long first = AXIS == 1 ? (i + 1) + (long long)n1 * (1 + (long long)n2 * (o + 1))
                                      : (i + 1) + (long long)n1 * ((o + 1) + (long long)n2);
    const float* line = src + first;
    float* out = dst + first;
    const long long vs = AXIS == 1 ? (long long)nx : (long long)nx * ny;
    const float* vline = AXIS == 1 ? V + i + (long long)nx * (ny + 1) * o : V + i + (long long)nx * o;
    float w0[7], w1[7], v[5];
    // T1[c0-3 .. c0+2] (ghosts at the line's start)
    {
        const int pf = c0 == 0 ? 0 : c0 - 3;  // first real T1 produced here
        const int np = c0 == 0 ? 3 : 6;       // how many
#pragma unroll
        for (int q = 0; q < 7; ++q) w0[q] = line_at<float>(line, stride, pf + q - 3, n, bc);
        float t1[6];
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            if (r < np) {
                const int pp = pf + r;
                t1[r] = weno_point_f32<QUIRK>(w0[0], w0[1], w0[2], w0[3], w0[4], w0[5], w0[6], vline[pp * vs],
                                              vline[(pp + 1) * vs], dt, h);
#pragma unroll
                for (int q = 0; q < 6; ++q) w0[q] = w0[q + 1];
                w0[6] = (pp + 1 < n) ? line_at<float>(line, stride, pp + 4, n, bc) : 0.f;
            } else {
                t1[r] = 0.f;
            }
        }
        if (c0 == 0) {
            w1[0] = weno_ghost(t1[2], true, bc);
            w1[1] = weno_ghost(t1[1], true, bc);
            w1[2] = weno_ghost(t1[0], true, bc);
            w1[3] = t1[0];
            w1[4] = t1[1];
            w1[5] = t1[2];
        } else {
#pragma unroll
            for (int q = 0; q < 6; ++q) w1[q] = t1[q];
        }
        // w0 = T0[c0 .. c0+6] now
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) v[q] = c0 + q <= n ? vline[(long long)(c0 + q) * vs] : 0.f;
    // difference windows: dw0[q] = h (w0[q+1] - w0[q]); dw1 likewise for w1[0..5]
    float dw0[6], dw1[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) dw0[q] = h * (w0[q + 1] - w0[q]);
#pragma unroll
    for (int q = 0; q < 5; ++q) dw1[q] = h * (w1[q + 1] - w1[q]);
#pragma unroll 2
    for (int c = c0; c < c1; ++c) {
        const int p = c + 3;  // T1 position entering the window
        float head;
        if (p < n) {
            head = weno_point_f32_d<QUIRK>(dw0, w0[2], w0[3], w0[5], v[3], v[4], dt, h);
        } else {
            // mirror 2n-1-p of T1 is in the window: w1[q] holds T1[c-3+q]
            const int q = 2 * n - 1 - p - (c - 3);
            float m = w1[5];
#pragma unroll
            for (int r = 0; r < 6; ++r)
                if (r == q) m = w1[r];
            head = weno_ghost(m, false, bc);
        }
        w1[6] = head;
        dw1[5] = h * (head - w1[5]);
        const float t = weno_point_f32_d<QUIRK>(dw1, w1[2], w1[3], w1[5], v[0], v[1], dt, h);
        out[(long long)c * stride] = 0.5f * t + 0.5f * w0[0];
#pragma unroll
        for (int q = 0; q < 6; ++q) w1[q] = w1[q + 1];
#pragma unroll
        for (int q = 0; q < 5; ++q) dw1[q] = dw1[q + 1];
#pragma unroll
        for (int q = 0; q < 6; ++q) w0[q] = w0[q + 1];
        w0[6] = (c + 4 < n) ? line_at<float>(line, stride, c + 7, n, bc) : 0.f;
#pragma unroll
        for (int q = 0; q < 5; ++q) dw0[q] = dw0[q + 1];
        dw0[5] = h * (w0[6] - w0[5]);
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = v[q + 1];
        v[4] = (c + 5 <= n) ? vline[(long long)(c + 5) * vs] : 0.f;
    }
}

// inner cells of a ghosted field: dst = src
__global__ void k_copy_inner_f32(float* __restrict__ dst, const float* __restrict__ src, int nx, int ny, int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= nx || j >= ny || k >= nz) return;
    const long long e = (i + 1) + (long long)(nx + 2) * ((j + 1) + (long long)(ny + 2) * (k + 1));
    dst[e] = src[e];
}

// One axis: cur is the field before the axis; returns the field after it
// (cur itself for in-place paths, `other` for the out-of-place march).
template <int AXIS, int QUIRK>
float* axis_f32(ht3d_ctx* ctx, float* cur, float* other, float* tmp, const float* V, float dt, float h, WenoBC bc,
                int nx, int ny, int nz) {
    const bool periodic = bc.typeL == HT3D_BC_PERIODIC || bc.typeR == HT3D_BC_PERIODIC;
    if (AXIS == 0) {
        const size_t smem = sizeof(float) * 2 * (size_t)(nx + 6) * kRowWarps;
        if (smem <= 96 * 1024) {
            if (smem > 48 * 1024)
                HT3D_CUDA(cudaFuncSetAttribute(k_weno_rows_f32<QUIRK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem));
            const long long rows = (long long)ny * nz;
            HT3D_LAUNCH(ctx, k_weno_rows_f32<QUIRK>, (unsigned)((rows + kRowWarps - 1) / kRowWarps), 32 * kRowWarps, smem,
                        cur, V, dt, h, bc, nx, ny, nz);
            return cur;
        }
    } else if (!periodic) {
        const int n = AXIS == 1 ? ny : nz;
        const dim3 g((nx + 127) / 128, AXIS == 1 ? nz : ny, (n + kMarchL - 1) / kMarchL);
        HT3D_LAUNCH(ctx, (k_weno_march_f32<AXIS, QUIRK>), g, 128, 0, cur, other, V, dt, h, bc, nx, ny, nz);
        return other;
    }
    dim3 b(32, 8, 1), g((nx + 31) / 32, (ny + 7) / 8, nz);
    HT3D_LAUNCH(ctx, (k_weno_stage_f32<AXIS, QUIRK, 1>), g, b, 0, cur, tmp, (const float*)nullptr, V, dt, h, bc, nx, ny,
                nz);
    HT3D_LAUNCH(ctx, (k_weno_stage_f32<AXIS, QUIRK, 2>), g, b, 0, tmp, cur, cur, V, dt, h, bc, nx, ny, nz);
    return cur;
}

template <int QUIRK>
void all_f32(ht3d_ctx* ctx, float* T, float* S, float* tmp, const float* const* V, float dt, const float* h,
             const WenoBC* bc, int nx, int ny, int nz) {
    float* cur = T;
    cur = axis_f32<0, QUIRK>(ctx, cur, cur == T ? S : T, tmp, V[0], dt, h[0], bc[0], nx, ny, nz);
    cur = axis_f32<1, QUIRK>(ctx, cur, cur == T ? S : T, tmp, V[1], dt, h[1], bc[1], nx, ny, nz);
    cur = axis_f32<2, QUIRK>(ctx, cur, cur == T ? S : T, tmp, V[2], dt, h[2], bc[2], nx, ny, nz);
    if (cur != T) {
        dim3 b(32, 8, 1), g((nx + 31) / 32, (ny + 7) / 8, nz);
        HT3D_LAUNCH(ctx, k_copy_inner_f32, g, b, 0, T, cur, nx, ny, nz);
    }
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
        float* S = (float*)ht3d_scratch(ctx, SLOT_AUX3, sizeof(float) * nex);   // out-of-place axis target
        float* tmp = (float*)ht3d_scratch(ctx, SLOT_AUX2, sizeof(float) * nex); // stage 1 of unfused axes
        const float* V[3] = {Vx, Vy, Vz};
        const float h[3] = {(float)_dx, (float)_dy, (float)_dz};
        if (variant == HT3D_WENO_V2_REF) all_f32<1>(ctx, Tc_ex, S, tmp, V, (float)dt, h, bc, nx, ny, nz);
        else all_f32<0>(ctx, Tc_ex, S, tmp, V, (float)dt, h, bc, nx, ny, nz);
        return HT3D_OK;
    });
}
