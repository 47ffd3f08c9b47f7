// WENO5 building blocks shared by the FP64/mixed sweeps (weno.cu) and the
// FP32 sweep (weno_f32.cu): the dFdx_Weno5! weights (tools/Weno5_Routines.jl:44-68)
// and the ghost rules of Boundaries_*_Weno5! evaluated on the fly.
#pragma once
#include "ht3d_internal.cuh"

namespace {

// ----------------------------------------------------------------- WENO core
// dFdx_Weno5! body, tools/Weno5_Routines.jl:51-66 (FP64, reference order)
__device__ __forceinline__ double weno5_ref(double v1, double v2, double v3, double v4, double v5) {
    const double p1 = v1 / 3.0 - 7.0 / 6.0 * v2 + 11.0 / 6.0 * v3;
    const double p2 = -v2 / 6.0 + 5.0 / 6.0 * v3 + v4 / 3.0;
    const double p3 = v3 / 3.0 + 5.0 / 6.0 * v4 - v5 / 6.0;
    const double maxV = fmax(fmax(fmax(fmax(v1 * v1, v2 * v2), v3 * v3), v4 * v4), v5 * v5);
    const double e = 1e-99 + 1e-6 * maxV;
    const double a1 = v1 - 2.0 * v2 + v3, b1 = v1 - 4.0 * v2 + 3.0 * v3;
    const double a2 = v2 - 2.0 * v3 + v4, b2 = v2 - v4;
    const double a3 = v3 - 2.0 * v4 + v5, b3 = 3.0 * v3 - 4.0 * v4 + v5;
    double w1 = 13.0 / 12.0 * (a1 * a1) + 1.0 / 4.0 * (b1 * b1);
    double w2 = 13.0 / 12.0 * (a2 * a2) + 1.0 / 4.0 * (b2 * b2);
    double w3 = 13.0 / 12.0 * (a3 * a3) + 1.0 / 4.0 * (b3 * b3);
    w1 = 0.1 / ((w1 + e) * (w1 + e));
    w2 = 0.6 / ((w2 + e) * (w2 + e));
    w3 = 0.3 / ((w3 + e) * (w3 + e));
    const double w = (w1 + w2 + w3);
    w1 = w1 / w;
    w2 = w2 / w;
    w3 = w3 / w;
    return w1 * p1 + w2 * p2 + w3 * p3;
}

// FP32 form for the mixed-precision path.  The reference's epsilon floor
// 1e-99 underflows in FP32; 1e-18 is the smallest floor whose square stays a
// normal FP32 number, so a flat field still yields the linear weights.
__device__ __forceinline__ float weno5_f32(float v1, float v2, float v3, float v4, float v5) {
    const float p1 = v1 * (1.0f / 3.0f) - (7.0f / 6.0f) * v2 + (11.0f / 6.0f) * v3;
    const float p2 = -v2 * (1.0f / 6.0f) + (5.0f / 6.0f) * v3 + v4 * (1.0f / 3.0f);
    const float p3 = v3 * (1.0f / 3.0f) + (5.0f / 6.0f) * v4 - v5 * (1.0f / 6.0f);
    // max of the squares = square of the largest magnitude (rounding is monotonic)
    const float vm = fmaxf(fmaxf(fmaxf(fmaxf(fabsf(v1), fabsf(v2)), fabsf(v3)), fabsf(v4)), fabsf(v5));
    const float maxV = vm * vm;
    const float e = 1e-18f + 1e-6f * maxV;
    const float a1 = v1 - 2.0f * v2 + v3, b1 = v1 - 4.0f * v2 + 3.0f * v3;
    const float a2 = v2 - 2.0f * v3 + v4, b2 = v2 - v4;
    const float a3 = v3 - 2.0f * v4 + v5, b3 = 3.0f * v3 - 4.0f * v4 + v5;
    const float s1 = (13.0f / 12.0f) * (a1 * a1) + 0.25f * (b1 * b1) + e;
    const float s2 = (13.0f / 12.0f) * (a2 * a2) + 0.25f * (b2 * b2) + e;
    const float s3 = (13.0f / 12.0f) * (a3 * a3) + 0.25f * (b3 * b3) + e;
    // approximate-reciprocal divisions (__fdividef, a few ulp): s >= 1e-18 keeps
    // every divisor and the weight sum (<= ~1e36) inside its accurate range
    const float w1 = __fdividef(0.1f, s1 * s1), w2 = __fdividef(0.6f, s2 * s2), w3 = __fdividef(0.3f, s3 * s3);
    return __fdividef(w1 * p1 + w2 * p2 + w3 * p3, w1 + w2 + w3);
}

// Mixed-precision form: the weighted sum of the three candidate stencils is
// rewritten as the central candidate plus weighted corrections,
//   w1 p1 + w2 p2 + w3 p3 = p2 + (w1 (p1 - p2) + w3 (p3 - p2)) / (w1 + w2 + w3),
// with p2 and the corrections (third differences) evaluated in FP64 from the
// FP64 differences v, and only the smoothness indicators and weights in FP32
// (from f, the same differences scaled and rounded to FP32).  A weight error
// then multiplies a correction, which is small wherever the field is smooth,
// instead of the derivative itself: FP32 weights cost ~1e-7 of the
// corrections, not ~1e-7 of the derivative.  v are unscaled differences; the
// caller multiplies the result by the grid factor h (f carry h already).
__device__ __forceinline__ double weno5_mixed(double v1, double v2, double v3, double v4, double v5, float f1,
                                              float f2, float f3, float f4, float f5) {
    const double p2 = __fma_rn(2.0, v4, __fma_rn(5.0, v3, -v2)) * (1.0 / 6.0);
    const float c1 = (float)(__fma_rn(3.0, v3 - v2, v1 - v4) * (1.0 / 3.0));  // p1 - p2
    const float c3 = (float)(__fma_rn(3.0, v4 - v3, v2 - v5) * (1.0 / 6.0));  // p3 - p2
    const float maxV = fmaxf(fmaxf(fmaxf(fmaxf(f1 * f1, f2 * f2), f3 * f3), f4 * f4), f5 * f5);
    const float e = 1e-18f + 1e-6f * maxV;
    const float a1 = f1 - 2.0f * f2 + f3, b1 = f1 - 4.0f * f2 + 3.0f * f3;
    const float a2 = f2 - 2.0f * f3 + f4, b2 = f2 - f4;
    const float a3 = f3 - 2.0f * f4 + f5, b3 = 3.0f * f3 - 4.0f * f4 + f5;
    const float s1 = (13.0f / 12.0f) * (a1 * a1) + 0.25f * (b1 * b1) + e;
    const float s2 = (13.0f / 12.0f) * (a2 * a2) + 0.25f * (b2 * b2) + e;
    const float s3 = (13.0f / 12.0f) * (a3 * a3) + 0.25f * (b3 * b3) + e;
    const float w1 = __fdividef(0.1f, s1 * s1), w2 = __fdividef(0.6f, s2 * s2), w3 = __fdividef(0.3f, s3 * s3);
    return p2 + (double)__fdividef(w1 * c1 + w3 * c3, w1 + w2 + w3);
}

// Upwinding multiplies each one-sided WENO5 derivative by a velocity factor
// that is exactly zero wherever the flow through that face has the other
// sign.  A derivative whose factor is zero is skipped (taken as 0): the
// product it would have added is a zero, so for finite fields the update
// T - dt*(Vp*dFm + Vm*dFp) keeps its value (at most the sign of a zero
// result differs), and where a warp's flow has one sign only one of the two
// reconstructions is evaluated.  The test reads the bit pattern (x != 0 for
// every input, NaN included), not an FP64 compare.
__device__ __forceinline__ bool upwind_active(double v) { return (__double_as_longlong(v) << 1) != 0; }
__device__ __forceinline__ bool upwind_active(float v) { return (__float_as_uint(v) << 1) != 0u; }

struct WenoBC {
    int typeL, typeR;
    double valL, valR;
};

// value at position p (-3 <= p <= n+2) along the sweep axis of a line whose
// inner value at index m is line[m*stride]; ghost rules of
// Boundaries_*_Weno5! (Neumann mirror, Dirichlet 2v-mirror, periodic wrap).
template <typename T>
__device__ __forceinline__ T line_at(const T* __restrict__ line, long long stride, int p, int n, const WenoBC& bc) {
    if (p < 0) {
        if (bc.typeL == HT3D_BC_PERIODIC) return line[(long long)(n + p) * stride];
        const T v = line[(long long)(-1 - p) * stride];
        return bc.typeL == HT3D_BC_DIRICHLET ? (T)(2 * bc.valL) - v : v;
    }
    if (p >= n) {
        if (bc.typeR == HT3D_BC_PERIODIC) return line[(long long)(p - n) * stride];
        const T v = line[(long long)(2 * n - 1 - p) * stride];
        return bc.typeR == HT3D_BC_DIRICHLET ? (T)(2 * bc.valR) - v : v;
    }
    return line[(long long)p * stride];
}


}  // namespace

// the mixed form's fused sweep on the march kernels (weno_f32.cu): the BCs as
// ht3d_weno5_advect takes them, none periodic
void ht3d_weno5_mixed_march(ht3d_ctx* ctx, double* T, double* S, const double* const* V, double dt, const double* h,
                            const int* bc_type6, const double* bc_val6, bool quirk, int nx, int ny, int nz);
