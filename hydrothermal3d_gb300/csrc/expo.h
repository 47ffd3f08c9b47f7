// exp(x) and 10^x in IEEE double, identical bits on the host (g++,
// -ffp-contract=off) and on the device (nvcc -fmad=false): only +, -, *, rint
// and exact power-of-two scalings, each rounded as written.  The material
// laws of the dimensional model (fluid viscosity 10^(247.8/(T-140)) and
// permeability exp(y/delta)) call these instead of the platform's libm or
// CUDA's exp/exp10, whose last bits differ between machines, so the device
// kernels and the CPU oracle evaluate the laws to the same bits.
//
// Method: Tang's table-driven exponential (ACM TOMS 15(2):144-157, 1989):
//   x = (32 m + j) L + r, L = ln2/32 (log10(2)/32 for 10^x), |r| <= L/2,
//   e^x = 2^m * 2^(j/32) * e^r,
// with the reduction constant split Cody-Waite style into a 32-bit head (exact
// products for |N| < 2^21) and a tail, 2^(j/32) tabulated as a double plus a
// correction, and e^r - 1 by its Taylor polynomial of degree 6 (truncation
// below 0.04 ulp for |r| <= ln2/64).  Error: below 1 ulp over the whole range
// (measured against 40-digit decimal arithmetic in the CPU tests).
// Constants: gen_expo.py (Python decimal arithmetic, 60 digits).
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define HT3D_EXPO_FN __host__ __device__ __forceinline__
#else
#define HT3D_EXPO_FN static inline
#endif

// BEGIN generated constants
// generated by gen_expo.py: do not edit
#define HT3D_EXPO_INV_L 0x1.71547652b82fep+5  // 32/ln2
#define HT3D_EXPO_L1 0x1.62e42fee00000p-6  // head of ln2/32 (32 bits)
#define HT3D_EXPO_L2 0x1.a39ef35793c76p-38  // ln2/32 - L1
#define HT3D_EXPO_INV_L10 0x1.a934f0979a371p+6  // 32 log2(10)
#define HT3D_EXPO_L10_1 0x1.3441350800000p-7  // head of log10(2)/32 (32 bits)
#define HT3D_EXPO_L10_2 0x1.f79fef311f12bp-39  // log10(2)/32 - L10_1
#define HT3D_EXPO_LN10 0x1.26bb1bbb55516p+1  // ln 10
#define HT3D_EXPO_A2 0x1.0000000000000p-1  // 1/2!
#define HT3D_EXPO_A3 0x1.5555555555555p-3  // 1/3!
#define HT3D_EXPO_A4 0x1.5555555555555p-5  // 1/4!
#define HT3D_EXPO_A5 0x1.1111111111111p-7  // 1/5!
#define HT3D_EXPO_A6 0x1.6c16c16c16c17p-10  // 1/6!
#define HT3D_EXPO_TABLE_HI \
    0x1.0000000000000p+0, 0x1.059b0d3158574p+0, 0x1.0b5586cf9890fp+0, 0x1.11301d0125b51p+0, \
    0x1.172b83c7d517bp+0, 0x1.1d4873168b9aap+0, 0x1.2387a6e756238p+0, 0x1.29e9df51fdee1p+0, \
    0x1.306fe0a31b715p+0, 0x1.371a7373aa9cbp+0, 0x1.3dea64c123422p+0, 0x1.44e086061892dp+0, \
    0x1.4bfdad5362a27p+0, 0x1.5342b569d4f82p+0, 0x1.5ab07dd485429p+0, 0x1.6247eb03a5585p+0, \
    0x1.6a09e667f3bcdp+0, 0x1.71f75e8ec5f74p+0, 0x1.7a11473eb0187p+0, 0x1.82589994cce13p+0, \
    0x1.8ace5422aa0dbp+0, 0x1.93737b0cdc5e5p+0, 0x1.9c49182a3f090p+0, 0x1.a5503b23e255dp+0, \
    0x1.ae89f995ad3adp+0, 0x1.b7f76f2fb5e47p+0, 0x1.c199bdd85529cp+0, 0x1.cb720dcef9069p+0, \
    0x1.d5818dcfba487p+0, 0x1.dfc97337b9b5fp+0, 0x1.ea4afa2a490dap+0, 0x1.f50765b6e4540p+0
#define HT3D_EXPO_TABLE_LO \
    0x0.0p+0, 0x1.d73e2a475b465p-55, 0x1.8a62e4adc610bp-54, -0x1.6c51039449b3ap-54, \
    -0x1.19041b9d78a76p-55, 0x1.e016e00a2643cp-54, 0x1.9b07eb6c70573p-54, 0x1.612e8afad1255p-55, \
    0x1.6f46ad23182e4p-55, -0x1.63aeabf42eae2p-54, 0x1.ada0911f09ebcp-55, 0x1.89b7a04ef80d0p-59, \
    0x1.d4397afec42e2p-56, -0x1.07abe1db13cadp-55, 0x1.6324c054647adp-54, -0x1.383c17e40b497p-54, \
    -0x1.bdd3413b26456p-54, -0x1.16e4786887a99p-55, -0x1.41577ee04992fp-55, -0x1.d4c1dd41532d8p-54, \
    0x1.6e9f156864b27p-54, -0x1.75fc781b57ebcp-57, 0x1.c7c46b071f2bep-56, -0x1.d2f6edb8d41e1p-54, \
    0x1.7a1cd345dcc81p-54, -0x1.5584f7e54ac3bp-56, 0x1.11065895048ddp-55, 0x1.503cbd1e949dbp-56, \
    0x1.2ed02d75b3707p-55, -0x1.1a5cd4f184b5cp-54, -0x1.e9c23179c2893p-54, 0x1.9d3e12dd8a18bp-54
// END generated constants

#if defined(__CUDACC__)
static __device__ const double ht3d_expo_hi_dev[32] = {HT3D_EXPO_TABLE_HI};
static __device__ const double ht3d_expo_lo_dev[32] = {HT3D_EXPO_TABLE_LO};
#endif
static const double ht3d_expo_hi_host[32] = {HT3D_EXPO_TABLE_HI};
static const double ht3d_expo_lo_host[32] = {HT3D_EXPO_TABLE_LO};

HT3D_EXPO_FN double ht3d_expo_from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
#endif
}

// 2^(j/32) (1 + p) 2^m for N = 32 m + j
HT3D_EXPO_FN double ht3d_expo_finish(int N, double p) {
    const int j = N & 31;
    const int m = (N - j) / 32;
#if defined(__CUDA_ARCH__)
    const double s_hi = ht3d_expo_hi_dev[j], s_lo = ht3d_expo_lo_dev[j];
#else
    const double s_hi = ht3d_expo_hi_host[j], s_lo = ht3d_expo_lo_host[j];
#endif
    const double q = s_hi + (s_lo + (s_hi + s_lo) * p);  // q in [0.98, 2.03)
    if (m > 1023) return q * ht3d_expo_from_bits((uint64_t)(m - 1 + 1023) << 52) * 2.0;
    if (m < -1021) return q * ht3d_expo_from_bits((uint64_t)(m + 54 + 1023) << 52) * 0x1p-54;
    return q * ht3d_expo_from_bits((uint64_t)(m + 1023) << 52);
}

// e^r - 1 for |r| <= ln2/64 (Taylor, degree 6, Horner)
HT3D_EXPO_FN double ht3d_expo_poly(double r1, double r2) {
    const double r = r1 + r2;
    const double q = r * r * (HT3D_EXPO_A2 + r * (HT3D_EXPO_A3 + r * (HT3D_EXPO_A4 + r * (HT3D_EXPO_A5 + r * HT3D_EXPO_A6))));
    return r1 + (r2 + q);
}

// e^x
HT3D_EXPO_FN double ht3d_exp(double x) {
    if (x != x) return x + x;
    if (x > 709.79) return ht3d_expo_from_bits(0x7ff0000000000000ull);
    if (x < -745.2) return 0.0;
    const double Nd = rint(x * HT3D_EXPO_INV_L);
    const double r1 = x - Nd * HT3D_EXPO_L1;  // exact
    const double r2 = -(Nd * HT3D_EXPO_L2);
    return ht3d_expo_finish((int)Nd, ht3d_expo_poly(r1, r2));
}

// 10^x
HT3D_EXPO_FN double ht3d_exp10(double x) {
    if (x != x) return x + x;
    if (x > 308.26) return ht3d_expo_from_bits(0x7ff0000000000000ull);
    if (x < -323.62) return 0.0;
    const double Nd = rint(x * HT3D_EXPO_INV_L10);
    const double r = (x - Nd * HT3D_EXPO_L10_1) - Nd * HT3D_EXPO_L10_2;  // |r| <= log10(2)/64
    const double s = r * HT3D_EXPO_LN10;                                   // |s| <= ln2/64
    return ht3d_expo_finish((int)Nd, ht3d_expo_poly(s, 0.0));
}
