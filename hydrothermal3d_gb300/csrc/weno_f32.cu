// WENO5 advection with FP32 storage and arithmetic: the same SSP-RK2
// dimension-split sweep as ht3d_weno5_advect (tools/Weno5_Routines.jl /
// tools/Weno5_Routines_v2.jl) on float fields, for the standalone sweep of
// the large-grid workload.  The epsilon floor of the weights is 1e-18 instead
// of 1e-99 (see weno5_f32).  Both stages of an axis run in one kernel: every
// thread marches along a segment of a line (register streams, below), along
// y and z straight from HBM with threads consecutive in x, along x over rows
// that a warp stages in shared memory.  Every axis reads T and V once and
// writes T once; periodic axes use the per-point kernels.
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

// ghost value at position p (< 0 or >= n) from its mirror value v
__device__ __forceinline__ float weno_ghost(float v, bool left, const WenoBC& bc) {
    const int t = left ? bc.typeL : bc.typeR;
    return t == HT3D_BC_DIRICHLET ? (float)(2 * (left ? bc.valL : bc.valR)) - v : v;
}

// Dirichlet/Neumann ends of an FP32 sweep: g = (float)(2 * value), so a ghost
// g - v rounds like the reference's 2 value - v evaluated in FP32.
struct WenoBCf {
    int typeL, typeR;
    float gL, gR;
};
__device__ __forceinline__ float weno_ghost(float v, bool left, const WenoBCf& bc) {
    const int t = left ? bc.typeL : bc.typeR;
    return t == HT3D_BC_DIRICHLET ? (left ? bc.gL : bc.gR) - v : v;
}
// FP64 ghost (the mixed form keeps T in FP64): 2 value - v in FP64
__device__ __forceinline__ double weno_ghost(double v, bool left, const WenoBC& bc) {
    const int t = left ? bc.typeL : bc.typeR;
    return t == HT3D_BC_DIRICHLET ? 2 * (left ? bc.valL : bc.valR) - v : v;
}

// --------------------------------------------------------------- streams
// A stream is the rolling state of one SSP-RK2 stage marching along a line:
// init() takes x_{i-3} .. x_{i+2} for the first point i, step() takes
// x_{i+3} and the velocities of the faces i (left) and i+1 (right), returns
// the stage value at i and advances to i+1.

// Face-shared form (WENO5 v1 stencil).  With one-sided differences
// D_j = h (x_{j+1} - x_j), every smoothness indicator of dFdx_Weno5!
// (tools/Weno5_Routines.jl:51-66) belongs to a triple (D_{j-1}, D_j, D_{j+1})
// with second difference a_j and spread c_j = D_{j-1} - D_{j+1}:
//   13/12 a^2 + 1/4 (2a - c)^2 = bC + a (a - c)   (first stencil,  "bL_j")
//   13/12 a^2 + 1/4 c^2        = bC               (central stencil, "bC_j")
//   13/12 a^2 + 1/4 (2a + c)^2 = bC + a (a + c)   (third stencil,  "bR_j")
// and reversing a triple swaps bL and bR, so
//   dF-(i) uses bL_{i-2}, bC_{i-1}, bR_i   and   dF+(i) uses bR_{i+1}, bC_i, bL_{i-1}.
// The weighted sum of the candidates is the central candidate p2 plus
// weighted third differences (p1 - p2 and p3 - p2), and those are differences
// of consecutive a:  g_j = a_j - a_{j-1}.  So each new face adds one triple
// (a, c, the three indicators, g) and one five-difference maximum e, and each
// point evaluates only its weights: the indicators are computed once per
// face instead of once per point and side.
struct WenoStreamShared {
    using value = float;      // storage and update type
    using bc_type = WenoBCf;  // its end rules
    using param = float;      // the grid factor h
    float x[6];   // x_{i-3} .. x_{i+2}
    float D[4];   // D_{i-2} .. D_{i+1}
    float bl[3];  // bL_{i-2} .. bL_i
    float bc[2];  // bC_{i-1}, bC_i
    float br;     // bR_i
    float g1[2];  // g_{i-1} / 3, g_i / 3
    float g3;     // g_i / 2
    float e;      // 1e-18 + 1e-6 max|D_{i-3} .. D_{i+1}|^2
    float ap;     // a_i
    float h;

    __device__ __forceinline__ static float rcp(float v) {
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
        return r;
    }
    // p2 + (w1 (p1 - p2) + w3 (p3 - p2)) / (w1 + w2 + w3) with w_k = d_k / s_k^2,
    // d = (0.1, 0.6, 0.3), all weights scaled by 10: n1 = p1 - p2, n3 = 3 (p3 - p2).
    // s >= 1e-18 keeps 1/s^2 <= 1e36 and the weight sum finite; |D| up to ~1e9
    // keeps it above the FP32 normal range.
    __device__ __forceinline__ static float mix(float b1, float b2, float b3, float e, float p2, float n1, float n3) {
        const float r1 = rcp(b1 + e), r2 = rcp(b2 + e), r3 = rcp(b3 + e);
        const float q1 = r1 * r1, q2 = r2 * r2, q3 = r3 * r3;
        const float W = fmaf(3.0f, q3, fmaf(6.0f, q2, q1));
        const float N = fmaf(q1, n1, q3 * n3);
        return fmaf(N, rcp(W), p2);
    }
    __device__ __forceinline__ static void triple(float Dm, float D0, float Dp, float& a, float& L, float& C,
                                                  float& R) {
        a = fmaf(-2.0f, D0, Dm) + Dp;
        const float c = Dm - Dp;
        C = fmaf(0.25f * c, c, (13.0f / 12.0f) * a * a);
        L = fmaf(a, a - c, C);
        R = fmaf(a, a + c, C);
    }
    __device__ __forceinline__ static float floor5(float d0, float d1, float d2, float d3, float d4) {
        const float m = fmaxf(fmaxf(fmaxf(fabsf(d0), fabsf(d1)), fmaxf(fabsf(d2), fabsf(d3))), fabsf(d4));
        return fmaf(1e-6f * m, m, 1e-18f);
    }

    __device__ __forceinline__ void init(const float (&x6)[6], float h_) {
        h = h_;
#pragma unroll
        for (int q = 0; q < 6; ++q) x[q] = x6[q];
        float d[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) d[q] = h * (x[q + 1] - x[q]);  // D_{i-3} .. D_{i+1}
        float a2, a1, a0, unused0, unused1, unused2;
        triple(d[0], d[1], d[2], a2, bl[0], unused0, unused1);   // centre i-2
        triple(d[1], d[2], d[3], a1, bl[1], bc[0], unused2);     // centre i-1
        triple(d[2], d[3], d[4], a0, bl[2], bc[1], br);          // centre i
        g1[0] = (a1 - a2) * (1.0f / 3.0f);
        g1[1] = (a0 - a1) * (1.0f / 3.0f);
        g3 = 0.5f * (a0 - a1);
        ap = a0;
        e = floor5(d[0], d[1], d[2], d[3], d[4]);
#pragma unroll
        for (int q = 0; q < 4; ++q) D[q] = d[q + 1];
    }

    __device__ __forceinline__ float back() const { return x[0]; }

    __device__ __forceinline__ float step(float xn, float va, float vb, float dt) {
        const float Dn = h * (xn - x[5]);  // D_{i+2}
        float a1, bL1, bC1, bR1;
        triple(D[2], D[3], Dn, a1, bL1, bC1, bR1);  // centre i+1
        const float g = a1 - ap;
        const float G1n = g * (1.0f / 3.0f), G3n = 0.5f * g;
        const float e1 = floor5(D[0], D[1], D[2], D[3], Dn);
        const float Vm = fminf(va, 0.0f), Vp = fmaxf(vb, 0.0f);
        float dFm = 0.0f, dFp = 0.0f;
        if (upwind_active(Vp)) {
            const float p2 = fmaf(5.0f / 6.0f, D[1], fmaf(1.0f / 3.0f, D[2], (-1.0f / 6.0f) * D[0]));
            dFm = mix(bl[0], bc[0], br, e, p2, -g1[0], -g3);
        }
        if (upwind_active(Vm)) {
            const float p2 = fmaf(5.0f / 6.0f, D[2], fmaf(1.0f / 3.0f, D[1], (-1.0f / 6.0f) * D[3]));
            dFp = mix(bR1, bc[1], bl[1], e1, p2, G1n, g3);
        }
        const float out = x[3] - dt * (Vp * dFm + Vm * dFp);
#pragma unroll
        for (int q = 0; q < 5; ++q) x[q] = x[q + 1];
        x[5] = xn;
#pragma unroll
        for (int q = 0; q < 3; ++q) D[q] = D[q + 1];
        D[3] = Dn;
        bl[0] = bl[1];
        bl[1] = bl[2];
        bl[2] = bL1;
        bc[0] = bc[1];
        bc[1] = bC1;
        br = bR1;
        g1[0] = g1[1];
        g1[1] = G1n;
        g3 = G3n;
        e = e1;
        ap = a1;
        return out;
    }
};

// Window form: the 7-point window and weno_point_f32, for the v2 stencil
// quirk (whose fifth difference of dF- spans three cells).
template <int QUIRK>
struct WenoStreamWindow {
    using value = float;
    using bc_type = WenoBCf;
    using param = float;
    float x[6];
    float h;
    __device__ __forceinline__ void init(const float (&x6)[6], float h_) {
        h = h_;
#pragma unroll
        for (int q = 0; q < 6; ++q) x[q] = x6[q];
    }
    __device__ __forceinline__ float back() const { return x[0]; }
    __device__ __forceinline__ float step(float xn, float va, float vb, float dt) {
        const float out = weno_point_f32<QUIRK>(x[0], x[1], x[2], x[3], x[4], x[5], xn, va, vb, dt, h);
#pragma unroll
        for (int q = 0; q < 5; ++q) x[q] = x[q + 1];
        x[5] = xn;
        return out;
    }
};

template <int QUIRK> struct StreamOf { using type = WenoStreamWindow<QUIRK>; };
template <> struct StreamOf<0> { using type = WenoStreamShared; };

// The upwind factors of an FP64 face velocity, v < 0 ? v : 0 and
// v >= 0 ? v : 0 (NaN gives 0), from the bit pattern: integer operations
// instead of two compares on the FP64 pipe.
__device__ __forceinline__ double neg_part(double v) {
    const long long b = __double_as_longlong(v);
    const unsigned long long m = (unsigned long long)b & 0x7fffffffffffffffULL;
    return (b < 0 && m != 0 && m <= 0x7ff0000000000000ULL) ? v : 0.0;
}
__device__ __forceinline__ double pos_part(double v) {
    const long long b = __double_as_longlong(v);
    const unsigned long long m = (unsigned long long)b & 0x7fffffffffffffffULL;
    return (m <= 0x7ff0000000000000ULL && (b >= 0 || m == 0)) ? v : 0.0;
}

// Mixed-precision form of the face-shared stream (the WENO5 stage of the
// mixed solver, weno5_mixed's split): T, the one-sided differences e (here
// unscaled, FP64), their second differences a and third differences g, and
// the central candidate p2 are FP64; the smoothness indicators, the floor and
// the weights are FP32 from the differences scaled by h and rounded; the
// weighted corrections (third differences, rounded to FP32) are added to p2
// in FP64, and the derivative is scaled by h.  Per new face: one FP64
// difference, one FP64 second and third difference, two conversions; per
// evaluation: p2 and one addition in FP64 (against six differences, six
// conversions and two corrections per point and side in the per-point form).
struct WenoStreamMixed {
    using value = double;
    using bc_type = WenoBC;
    using param = double;
    double x[6];  // x_{i-3} .. x_{i+2}
    double E[4];  // e_{i-2} .. e_{i+1} (e_j = x_{j+1} - x_j)
    double ap;    // a_i
    float D[4];   // h e, rounded to FP32, same faces
    float bl[3], bc[2], br, g1[2], g3, e;
    float hf;
    double h;

    __device__ __forceinline__ void init(const double (&x6)[6], double h_) {
        h = h_;
        hf = (float)h_;
#pragma unroll
        for (int q = 0; q < 6; ++q) x[q] = x6[q];
        double ee[5];
        float d[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            ee[q] = x[q + 1] - x[q];  // e_{i-3} .. e_{i+1}
            d[q] = hf * (float)ee[q];
        }
        float a2, a1, a0, u0, u1, u2;
        WenoStreamShared::triple(d[0], d[1], d[2], a2, bl[0], u0, u1);
        WenoStreamShared::triple(d[1], d[2], d[3], a1, bl[1], bc[0], u2);
        WenoStreamShared::triple(d[2], d[3], d[4], a0, bl[2], bc[1], br);
        const double A2 = __fma_rn(-2.0, ee[1], ee[0]) + ee[2];  // a_{i-2}
        const double A1 = __fma_rn(-2.0, ee[2], ee[1]) + ee[3];  // a_{i-1}
        const double A0 = __fma_rn(-2.0, ee[3], ee[2]) + ee[4];  // a_i
        const float gm = (float)(A1 - A2), g0 = (float)(A0 - A1);
        g1[0] = gm * (1.0f / 3.0f);
        g1[1] = g0 * (1.0f / 3.0f);
        g3 = 0.5f * g0;
        ap = A0;
        e = WenoStreamShared::floor5(d[0], d[1], d[2], d[3], d[4]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            E[q] = ee[q + 1];
            D[q] = d[q + 1];
        }
    }

    __device__ __forceinline__ double back() const { return x[0]; }

    __device__ __forceinline__ double step(double xn, double va, double vb, double dt) {
        const double en = xn - x[5];  // e_{i+2}
        const float Dn = hf * (float)en;
        float af, bL1, bC1, bR1;
        WenoStreamShared::triple(D[2], D[3], Dn, af, bL1, bC1, bR1);  // centre i+1 (indicators)
        const double a1 = __fma_rn(-2.0, E[3], E[2]) + en;            // a_{i+1}
        const float gf = (float)(a1 - ap);                            // g_{i+1}
        const float G1n = gf * (1.0f / 3.0f), G3n = 0.5f * gf;
        const float e1 = WenoStreamShared::floor5(D[0], D[1], D[2], D[3], Dn);
        const double Vm = neg_part(va), Vp = pos_part(vb);
        double rhs = 0.0;  // Vp dF- + Vm dF+ (unscaled derivatives)
        if (upwind_active(Vp)) {
            const double p2 = __fma_rn(2.0, E[2], __fma_rn(5.0, E[1], -E[0])) * (1.0 / 6.0);
            rhs = Vp * (p2 + (double)WenoStreamShared::mix(bl[0], bc[0], br, e, 0.0f, -g1[0], -g3));
        }
        if (upwind_active(Vm)) {
            const double p2 = __fma_rn(2.0, E[1], __fma_rn(5.0, E[2], -E[3])) * (1.0 / 6.0);
            rhs = __fma_rn(Vm, p2 + (double)WenoStreamShared::mix(bR1, bc[1], bl[1], e1, 0.0f, G1n, g3), rhs);
        }
        const double out = __fma_rn(-(dt * h), rhs, x[3]);  // dt h: loop invariant
#pragma unroll
        for (int q = 0; q < 5; ++q) x[q] = x[q + 1];
        x[5] = xn;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            E[q] = E[q + 1];
            D[q] = D[q + 1];
        }
        E[3] = en;
        D[3] = Dn;
        bl[0] = bl[1];
        bl[1] = bl[2];
        bl[2] = bL1;
        bc[0] = bc[1];
        bc[1] = bC1;
        br = bR1;
        g1[0] = g1[1];
        g1[1] = G1n;
        g3 = G3n;
        e = e1;
        ap = a1;
        return out;
    }
};

// Mixed form from the 7-point window (weno5_mixed per point and side), for
// the v2 stencil quirk.
template <int QUIRK>
struct WenoStreamMixedWindow {
    using value = double;
    using bc_type = WenoBC;
    using param = double;
    double x[6];
    double h;
    __device__ __forceinline__ void init(const double (&x6)[6], double h_) {
        h = h_;
#pragma unroll
        for (int q = 0; q < 6; ++q) x[q] = x6[q];
    }
    __device__ __forceinline__ double back() const { return x[0]; }
    __device__ __forceinline__ double step(double xn, double va, double vb, double dt) {
        const double Vm = va < 0.0 ? va : 0.0;
        const double Vp = vb >= 0.0 ? vb : 0.0;
        const float hf = (float)h;
        double e[6];
        float f[6];
#pragma unroll
        for (int o = 0; o < 5; ++o) e[o] = x[o + 1] - x[o];
        e[5] = xn - x[5];
#pragma unroll
        for (int o = 0; o < 6; ++o) f[o] = hf * (float)e[o];
        const double e5 = QUIRK ? x[5] - x[2] : e[4];
        const float f5 = QUIRK ? hf * (float)e5 : f[4];
        const double dFm = upwind_active(Vp) ? weno5_mixed(e[0], e[1], e[2], e[3], e5, f[0], f[1], f[2], f[3], f5)
                                             : 0.0;
        const double dFp = upwind_active(Vm)
                               ? weno5_mixed(e[5], e[4], e[3], e[2], e[1], f[5], f[4], f[3], f[2], f[1])
                               : 0.0;
        const double out = x[3] - dt * (h * (Vp * dFm + Vm * dFp));
#pragma unroll
        for (int q = 0; q < 5; ++q) x[q] = x[q + 1];
        x[5] = xn;
        return out;
    }
};
template <int QUIRK> struct MixedStreamOf { using type = WenoStreamMixedWindow<QUIRK>; };
template <> struct MixedStreamOf<0> { using type = WenoStreamMixed; };

// ------------------------------------------------------------------ march
// Both stages along the segment [c0, c1) of a line of n cells (Neumann or
// Dirichlet ends, n >= 3, c1 - c0 >= 3, c0 == 0 or c0 >= 8).  Stage 1 runs
// three points ahead of stage 2: it starts at c0 - 3 (for c0 == 0 the three
// points before the line are replaced by the mirror rule after the stage,
// like Boundaries_*_Weno5!), and each step produces T1[c + 3] and then
// T[c] = (T0[c] + stage2(T1)[c]) / 2.  Near the line's end T1 beyond it is the
// mirror of the last three T1 values.


template <class Stream>
struct March {
    using T = typename Stream::value;
    using BC = typename Stream::bc_type;
    Stream s1, s2;
    T v0, v1, v2, v3;  // faces c .. c + 3 of the next step
    T gq0, gq1, gq2;   // tail: the T1 ghosts n, n + 1, n + 2
    T tq0, tq1, tq2;   // tail: T0[n - 3 .. n - 1]

    //   src.t0(q): T0 at q in [c0 - 6, c0 + 6) (ghosts by the BC rule; positions
    //              before -3 only feed discarded points: any finite value)
    //   src.v(f):  face f in [c0 - 3, c0 + 3] (faces < 0: any finite value)
    template <class Src>
    __device__ __forceinline__ void start(const Src& src, int c0, const BC& bc, T dt, typename Stream::param h) {
        {
            T x[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) x[q] = src.t0(c0 - 6 + q);
            s1.init(x, h);
        }
        T w[6];  // T1[c0 - 3 .. c0 + 2]
#pragma unroll
        for (int r = 0; r < 6; ++r) w[r] = s1.step(src.t0(c0 + r), src.v(c0 - 3 + r), src.v(c0 - 2 + r), dt);
        if (c0 == 0) {
            w[0] = weno_ghost(w[5], true, bc);
            w[1] = weno_ghost(w[4], true, bc);
            w[2] = weno_ghost(w[3], true, bc);
        }
        s2.init(w, h);
        v0 = src.v(c0);
        v1 = src.v(c0 + 1);
        v2 = src.v(c0 + 2);
        v3 = src.v(c0 + 3);
    }
    // step c with its stage-1 point c + 3 inside the line: xa = T0[c + 6]
    // (a ghost past the end), va = face c + 4; returns T[c]
    __device__ __forceinline__ T step(T xa, T va, T dt) {
        const T t0c = s1.back();  // T0[c]
        const T t1 = s1.step(xa, v3, va, dt);
        const T t = s2.step(t1, v0, v1, dt);
        v0 = v1;
        v1 = v2;
        v2 = v3;
        v3 = va;
        return (T)0.5 * t + (T)0.5 * t0c;
    }
    // at c = n - 3: s1 holds T0[n - 3 .. n + 2], s2 T1[n - 6 .. n - 1]
    __device__ __forceinline__ void tail_enter(const BC& bc) {
        tq0 = s1.x[0];
        tq1 = s1.x[1];
        tq2 = s1.x[2];
        gq0 = weno_ghost(s2.x[5], false, bc);
        gq1 = weno_ghost(s2.x[4], false, bc);
        gq2 = weno_ghost(s2.x[3], false, bc);
    }
    __device__ __forceinline__ T tail_step(T dt) {  // c = n - 3, n - 2, n - 1 in turn
        const T t = s2.step(gq0, v0, v1, dt);
        const T out = (T)0.5 * t + (T)0.5 * tq0;
        gq0 = gq1;
        gq1 = gq2;
        tq0 = tq1;
        tq1 = tq2;
        v0 = v1;
        v1 = v2;
        v2 = v3;
        return out;
    }
};

// y or z line straight from HBM (out of place: src -> dst, the inner cells);
// the read-only loads may move ahead of the stores of earlier steps.
template <class T, class BC>
struct LineSrc {
    const T* line;  // inner cell 0 of the line
    T* out;
    const T* vline;  // face 0
    long long stride, vs;
    int n;
    BC bc;
    __device__ __forceinline__ T ld(int q) const { return __ldg(line + (long long)q * stride); }
    __device__ __forceinline__ T t0(int q) const {
        if (q >= 0 && q < n) return ld(q);
        if (q < -3) return (T)0;
        return q < 0 ? weno_ghost(ld(-1 - q), true, bc) : weno_ghost(ld(2 * n - 1 - q), false, bc);
    }
    __device__ __forceinline__ T v(int f) const { return f >= 0 ? __ldg(vline + (long long)f * vs) : (T)0; }
    __device__ __forceinline__ void put(int c, T val) const { out[(long long)c * stride] = val; }
};

// Balanced segments: kMarchL cells per thread on average, at least 48 each
// when a line has more than one.
constexpr int kMarchL = 64;
constexpr int kMarchUnroll = 4;  // steps per software-pipelined body of the y/z march
__host__ __device__ __forceinline__ int march_chunks(int n) { return n < 3 * kMarchL / 2 ? 1 : (n + kMarchL / 2) / kMarchL; }

template <int AXIS, class Stream>
__global__ void __launch_bounds__(128) k_weno_march(const typename Stream::value* __restrict__ src,
                                                    typename Stream::value* __restrict__ dst,
                                                    const typename Stream::value* __restrict__ V,
                                                    typename Stream::value dt, typename Stream::param h,
                                                    typename Stream::bc_type bc, int nx, int ny, int nz) {
    using T = typename Stream::value;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int o = blockIdx.y;  // k for the y-march, j for the z-march
    const int n = AXIS == 1 ? ny : nz;
    const int K = march_chunks(n);
    const int c0 = (int)((long long)blockIdx.z * n / K), c1 = (int)((long long)(blockIdx.z + 1) * n / K);
    if (i >= nx) return;
    const int n1 = nx + 2, n2 = ny + 2;
    LineSrc<T, typename Stream::bc_type> s;
    s.stride = AXIS == 1 ? (long long)n1 : (long long)n1 * n2;
    const long long first = AXIS == 1 ? (i + 1) + (long long)n1 * (1 + (long long)n2 * (o + 1))
                                      : (i + 1) + (long long)n1 * ((o + 1) + (long long)n2);
    s.line = src + first;
    s.out = dst + first;
    s.vs = AXIS == 1 ? (long long)nx : (long long)nx * ny;
    s.vline = AXIS == 1 ? V + i + (long long)nx * (ny + 1) * o : V + i + (long long)nx * o;
    s.n = n;
    s.bc = bc;
    March<Stream> M;
    M.start(s, c0, bc, dt, h);
    const int cA = c1 < n ? c1 : n - 3;  // steps whose stage-1 point c + 3 is inside the line
    const int cB = min(cA, n - 6);       // ... and whose T0[c + 6] is too
    int c = c0;
    if (cB - c0 >= 2 * kMarchUnroll) {
        // software pipeline: the T0 and face values of the next kMarchUnroll
        // steps are loaded while the current ones compute
        T qt[kMarchUnroll], qv[kMarchUnroll];
#pragma unroll
        for (int u = 0; u < kMarchUnroll; ++u) {
            qt[u] = s.ld(c + 6 + u);
            qv[u] = s.v(c + 4 + u);
        }
        for (; c + 2 * kMarchUnroll <= cB; c += kMarchUnroll) {
            T nt[kMarchUnroll], nv[kMarchUnroll];
#pragma unroll
            for (int u = 0; u < kMarchUnroll; ++u) {
                nt[u] = s.ld(c + kMarchUnroll + 6 + u);  // < cB + 6 <= n
                nv[u] = s.v(c + kMarchUnroll + 4 + u);
            }
#pragma unroll
            for (int u = 0; u < kMarchUnroll; ++u) s.put(c + u, M.step(qt[u], qv[u], dt));
#pragma unroll
            for (int u = 0; u < kMarchUnroll; ++u) {
                qt[u] = nt[u];
                qv[u] = nv[u];
            }
        }
#pragma unroll
        for (int u = 0; u < kMarchUnroll; ++u) s.put(c + u, M.step(qt[u], qv[u], dt));
        c += kMarchUnroll;
    }
    for (; c < cB; ++c) s.put(c, M.step(s.ld(c + 6), s.v(c + 4), dt));
    for (; c < cA; ++c) s.put(c, M.step(s.t0(c + 6), s.v(c + 4), dt));
    if (c1 == n) {
        M.tail_enter(bc);
#pragma unroll
        for (int r = 0; r < 3; ++r) s.put(n - 3 + r, M.tail_step(dt));
    }
}

// x: a warp marches 32 consecutive rows (one per lane) along x.
// T0 and Vx reach shared memory through per-row rings of three 8-cell tiles,
// filled by asynchronous element-size copies one tile ahead of the march; a
// step reads its own row's ring (odd row pitch: the 32 lanes hit 32 banks,
// 8-byte elements 16 bank pairs per half-warp) and
// leaves T[c] in the slot of T0[c], which the warp then stores coalesced.
// Tile u of a segment holds positions b0 + 8u .. b0 + 8u + 7 (b0 = c0 - 8)
// in ring slot u % 3; the steps c0 + 8v .. c0 + 8v + 7 (block v) read tiles
// v + 1 and v + 2 and write tile v + 1.
constexpr int kXW = 8;
constexpr int kXPitch = 3 * kXW + 1;
// warps per block: the rings of one warp take 12.8 KB of 8-byte elements
template <class T> struct XWarps { static constexpr int value = sizeof(T) == 4 ? 4 : 2; };

template <class T>
__device__ __forceinline__ void cp_async_el(T* dst, const T* src) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src),
                 "n"((int)sizeof(T))
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <class T, class BC>
struct RingSrc {
    T* t;         // this lane's row of the T0 ring
    const T* vp;  // ... of the Vx ring
    int b0, n;
    BC bc;
    __device__ __forceinline__ int col(int q) const {
        const int d = q - b0;
        return ((d >> 3) % 3) * kXW + (d & 7);
    }
    __device__ __forceinline__ T t0(int q) const {
        if (q >= 0 && q < n) return t[col(q)];
        if (q < -3) return (T)0;
        return q < 0 ? weno_ghost(t[col(-1 - q)], true, bc) : weno_ghost(t[col(2 * n - 1 - q)], false, bc);
    }
    __device__ __forceinline__ T v(int f) const { return f >= 0 ? vp[col(f)] : (T)0; }
    __device__ __forceinline__ void put(int c, T val) const { t[col(c)] = val; }
};

// The x sweep updates T in place, so a row is never split between warps:
// a segment's halo (six cells on each side) would be the neighbouring
// segment's cells, which another block may already have overwritten.  Within
// a warp the ring's copies run ahead of its stores (tile v + 4 is fetched
// after tile v + 1 is stored), so whole rows are safe.
template <class Stream>
__global__ void __launch_bounds__(32 * XWarps<typename Stream::value>::value)
    k_weno_xstream(typename Stream::value* __restrict__ T, const typename Stream::value* __restrict__ Vx,
                   typename Stream::value dt, typename Stream::param h, typename Stream::bc_type bc, int nx, int ny,
                   int nz) {
    using E = typename Stream::value;
    constexpr int kXWarps = XWarps<E>::value;
    __shared__ E ring[kXWarps][2][32 * kXPitch];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long rows = (long long)ny * nz;
    const long long row0 = ((long long)blockIdx.x * kXWarps + warp) * 32;
    if (row0 >= rows) return;  // whole warps only
    const int n = nx;
    const int c0 = 0, c1 = n;  // whole rows (see above)
    const int b0 = c0 - kXW;
    E* tr = ring[warp][0];
    E* vr = ring[warp][1];
    // copy lanes: column lane & 7 of rows sub + 4 k (k = 0 .. 7), rows past the
    // last one read the last row and store nothing
    const int sub = lane >> 3, cc = lane & 7;
    const long long rlast = rows - 1;
    const long long tbase = 1 + (long long)(nx + 2) * (1 + (long long)(ny + 2));  // inner cell 0 of row 0
    unsigned rel[8];                                                              // row offsets from row0's
    long long t0off;
    {
        const long long r0 = row0;
        t0off = tbase + (long long)(nx + 2) * (r0 + 2 * (r0 / ny));
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long r = min(row0 + sub + 4 * k, rlast);
            rel[k] = (unsigned)(tbase + (long long)(nx + 2) * (r + 2 * (r / ny)) - t0off);
        }
    }
    const E* Tw = T + t0off;
    const E* Vw = Vx + (long long)(nx + 1) * row0;
    const int tq_lo = max(0, c0 - 6), tq_hi = min(n, c1 + 6);  // T0 positions a segment reads
    const int vq_lo = max(0, c0 - 3), vq_hi = min(n, c1 + 3);  // faces (inclusive)
    auto load_tile = [&](int u) {
        const int q = b0 + kXW * u + cc;
        E* td = tr + (u % 3) * kXW + cc;
        E* vd = vr + (u % 3) * kXW + cc;
        const bool tq = q >= tq_lo && q < tq_hi, vq = q >= vq_lo && q <= vq_hi;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int r = sub + 4 * k;
            const long long rv = min(row0 + r, rlast) - row0;
            if (tq) cp_async_el(td + r * kXPitch, Tw + rel[k] + q);
            if (vq) cp_async_el(vd + r * kXPitch, Vw + (nx + 1) * rv + q);
        }
        cp_async_commit();
    };
    auto store_tile = [&](int u, int lo, int hi) {  // positions [lo, hi) of tile u
        const int q = b0 + kXW * u + cc;
        if (q < lo || q >= hi) return;
        const E* ts = tr + (u % 3) * kXW + cc;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int r = sub + 4 * k;
            if (row0 + r <= rlast) T[t0off + rel[k] + q] = ts[r * kXPitch];
        }
    };
    load_tile(0);
    load_tile(1);
    load_tile(2);
    cp_async_wait<0>();
    __syncwarp();
    RingSrc<E, typename Stream::bc_type> src;
    src.t = tr + lane * kXPitch;
    src.vp = vr + lane * kXPitch;
    src.b0 = b0;
    src.n = n;
    src.bc = bc;
    March<Stream> M;
    M.start(src, c0, bc, dt, h);
    __syncwarp();
    load_tile(3);
    const int cA = c1 < n ? c1 : n - 3;
    for (int v = 0, cb = c0; cb < c1; ++v, cb += kXW) {
        E* tcur = src.t + ((v + 1) % 3) * kXW;  // positions cb .. cb + 7
        const E* tnxt = src.t + ((v + 2) % 3) * kXW;
        const E* vcur = src.vp + ((v + 1) % 3) * kXW;
        const E* vnxt = src.vp + ((v + 2) % 3) * kXW;
        if (cb + kXW <= cA && cb + kXW + 6 <= n) {  // eight steps without ghosts
#pragma unroll
            for (int m = 0; m < kXW; ++m) {
                const E xa = m + 6 < kXW ? tcur[m + 6] : tnxt[m + 6 - kXW];
                const E va = m + 4 < kXW ? vcur[m + 4] : vnxt[m + 4 - kXW];
                tcur[m] = M.step(xa, va, dt);
            }
        } else {
            for (int m = 0; m < kXW && cb + m < c1; ++m) {
                const int c = cb + m;
                E out;
                if (c < cA) {
                    out = M.step(src.t0(c + 6), src.v(c + 4), dt);
                } else {
                    if (c == n - 3) M.tail_enter(bc);
                    out = M.tail_step(dt);
                }
                src.put(c, out);
            }
        }
        __syncwarp();
        store_tile(v + 1, c0, c1);
        load_tile(v + 4);  // into the slot just stored
        cp_async_wait<1>();
        __syncwarp();
    }
    cp_async_wait<0>();
}

// Row-at-a-time x kernel for periodic x: a warp owns a row; the row of T0 and
// of the stage-1 result T1 live in shared memory with three ghost cells on
// each side (filled by the BC rules after each stage).
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

// inner cells of a ghosted field: dst = src
__global__ void k_copy_inner_f32(float* __restrict__ dst, const float* __restrict__ src, int nx, int ny, int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= nx || j >= ny || k >= nz) return;
    const long long e = (i + 1) + (long long)(nx + 2) * ((j + 1) + (long long)(ny + 2) * (k + 1));
    dst[e] = src[e];
}

WenoBCf bcf(const WenoBC& b) {
    return WenoBCf{b.typeL, b.typeR, (float)(2 * b.valL), (float)(2 * b.valR)};
}

// One axis: cur is the field before the axis; returns the field after it
// (cur itself for in-place paths, `other` for the out-of-place march).
template <int AXIS, int QUIRK>
float* axis_f32(ht3d_ctx* ctx, float* cur, float* other, float* tmp, const float* V, float dt, float h, WenoBC bc,
                int nx, int ny, int nz) {
    const bool periodic = bc.typeL == HT3D_BC_PERIODIC || bc.typeR == HT3D_BC_PERIODIC;
    if constexpr (AXIS == 0) {
        if (!periodic) {
            using S = typename StreamOf<QUIRK>::type;
            constexpr int warps = XWarps<float>::value;
            const long long rows = (long long)ny * nz, per_block = 32LL * warps;
            const dim3 g((unsigned)((rows + per_block - 1) / per_block));
            HT3D_LAUNCH(ctx, k_weno_xstream<S>, g, 32 * warps, 0, cur, V, dt, h, bcf(bc), nx, ny, nz);
            return cur;
        }
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
    } else {
        if (!periodic) {
            const int n = AXIS == 1 ? ny : nz;
            const dim3 g((nx + 127) / 128, AXIS == 1 ? nz : ny, march_chunks(n));
            HT3D_LAUNCH(ctx, (k_weno_march<AXIS, typename StreamOf<QUIRK>::type>), g, 128, 0, cur, other, V, dt, h,
                        bcf(bc), nx, ny, nz);
            return other;
        }
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

// The mixed form's fused sweep (FP64 T, mixed stencils): x in place, y T -> S,
// z S -> T, every axis one launch (both stages).
template <int QUIRK>
void all_mixed(ht3d_ctx* ctx, double* T, double* S, const double* const* V, double dt, const double* h,
               const WenoBC* bc, int nx, int ny, int nz) {
    using St = typename MixedStreamOf<QUIRK>::type;
    constexpr int warps = XWarps<double>::value;
    const long long rows = (long long)ny * nz, per_block = 32LL * warps;
    HT3D_LAUNCH(ctx, k_weno_xstream<St>, (unsigned)((rows + per_block - 1) / per_block), 32 * warps, 0, T, V[0], dt,
                h[0], bc[0], nx, ny, nz);
    HT3D_LAUNCH(ctx, (k_weno_march<1, St>), dim3((nx + 127) / 128, nz, march_chunks(ny)), 128, 0, T, S, V[1], dt,
                h[1], bc[1], nx, ny, nz);
    HT3D_LAUNCH(ctx, (k_weno_march<2, St>), dim3((nx + 127) / 128, ny, march_chunks(nz)), 128, 0, S, T, V[2], dt,
                h[2], bc[2], nx, ny, nz);
}

}  // namespace

// Mixed-form WENO5 sweep through the march kernels (weno.cu calls it when no
// axis is periodic; S: an FP64 field of the ghosted size for the y axis).
void ht3d_weno5_mixed_march(ht3d_ctx* ctx, double* T, double* S, const double* const* V, double dt, const double* h,
                            const int* bc_type6, const double* bc_val6, bool quirk, int nx, int ny, int nz) {
    WenoBC bc[3];
    for (int a = 0; a < 3; ++a) bc[a] = WenoBC{bc_type6[2 * a], bc_type6[2 * a + 1], bc_val6[2 * a], bc_val6[2 * a + 1]};
    if (quirk) all_mixed<1>(ctx, T, S, V, dt, h, bc, nx, ny, nz);
    else all_mixed<0>(ctx, T, S, V, dt, h, bc, nx, ny, nz);
}

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
