// Fluid and rock laws of Dimensional/HydroThermal3D_v18.jl:29-39, with the
// reference's evaluation order (include from -fmad=false translation units).
// x^2 and x^3 are products as Julia's literal powers; x^4 is (x^2)^2.
#pragma once
#include "expo.h"

__host__ __device__ inline double law_kTs(double T) { return 3.1138 - 0.0023 * (T); }
__host__ __device__ inline double law_kTf(double T) { return -0.069 + 0.0012 * (T); }
__host__ __device__ inline double law_Cf(double T) { return 1000 + 7.5 * (T); }
__host__ __device__ inline double law_Cs(double T) { return 0.5915 * (T) + 636.14; }
__host__ __device__ inline double law_rhos(double T) { return 2800 * (1 - (0.000024 * (T - 293))); }
__host__ __device__ inline double law_rhof_C(double T_C, double p) {
    const double p2 = p * p, p3 = p * p * p, p4 = p2 * p2, T2 = T_C * T_C, T3 = T_C * T_C * T_C, T4 = T2 * T2;
    return 1006 + (7.424e-7 * p) + (-0.3922 * T_C) + (-4.441e-15 * p2) + (4.547e-9 * p * T_C) + (-0.003774 * T2) +
           (1.451e-23 * p3) + (-1.793e-17 * p2 * T_C) + (7.485e-12 * p * T2) + (2.955e-6 * T3) + (-1.463e-32 * p4) +
           (1.361e-26 * p3 * T_C) + (4.018e-21 * (p2) * (T2)) + (-7.372e-15 * p * T3) + (5.698e-11 * T4);
}
__host__ __device__ inline double law_drhodP_C(double T_C, double p) {
    const double T2 = T_C * T_C, T3 = T_C * T_C * T_C, p2 = p * p, p3 = p * p * p;
    return -7.372e-15 * T3 + 8.036e-21 * T2 * p + 7.485e-12 * T2 + 4.083e-26 * T_C * p2 - 3.586e-17 * T_C * p +
           4.547e-9 * T_C - 5.852e-32 * p3 + 4.353e-23 * p2 - 8.882e-15 * p + 7.424e-7;
}
// 10^x and e^x: ht3d_exp10/ht3d_exp (expo.h), one implementation whose bits
// are the same on the device and in the host's CPU oracle
__host__ __device__ inline double law_muf(double T) { return 2.414e-5 * ht3d_exp10(247.8 / (T - 140.)); }
__host__ __device__ inline double law_kF(double y, double delta) { return 5e-16 * ht3d_exp(y / delta); }
__host__ __device__ inline double law_phi(double phase, double phi0) { return phase == 2.0 ? 3 * phi0 : phi0; }

// index: 0 kTs, 1 kTf, 2 Cf, 3 Cs, 4 rhos, 5 rhof_C(T_C,p), 6 drhodP_C(T_C,p), 7 muf, 8 kF(y,delta), 9 phi(phase,phi0),
// 10 e^a, 11 10^a (the exponentials the laws use)
__host__ __device__ inline double law_eval(int which, double a, double b) {
    switch (which) {
        case 0: return law_kTs(a);
        case 1: return law_kTf(a);
        case 2: return law_Cf(a);
        case 3: return law_Cs(a);
        case 4: return law_rhos(a);
        case 5: return law_rhof_C(a, b);
        case 6: return law_drhodP_C(a, b);
        case 7: return law_muf(a);
        case 8: return law_kF(a, b);
        case 9: return law_phi(a, b);
        case 10: return ht3d_exp(a);
        case 11: return ht3d_exp10(a);
    }
    return 0.0;
}
