// Fused DYREL solver for the dimensionless diffusion problems of the
// HydroThermal3D hot path.
//
// One launch of k_dyrel_iter performs one pseudo-iteration of the reference
// loop Dimensional/HydroThermal3D_v18.jl:448-455 composed with the
// dimensionless residual:
//     SetFaceBCs(X) ; ComputeFlux!(q, k, X) ;
//     F = (R + cX*inn(X) + div q) / PC ;  DYRELUpdate!(F0, X, F, h1, h2, dtau)
// reading every field once.  Ghost cells are evaluated on the fly from the
// adjacent inner cell; the updated field goes to a second buffer (ping-pong),
// so every thread sees the pre-iteration state exactly like the reference's
// separate launches do.  The output buffer's face ghosts receive BC(X_in),
// which is the state the reference leaves after the same iteration.
//
// Two thread layouts with identical arithmetic (selected per context):
//  * k_dyrel_iter: a 32x8 tile of (x,y) columns per block marching in z over a
//    chunk of planes, the z-face flux carried in a register;
//  * k_dyrel_cell: one thread per cell, neighbours through L1/L2.
#pragma once
#include <type_traits>
#include "ht3d_internal.cuh"

namespace {

struct DyrelScal {
    double h1, h2, dtau, cX, _dx, _dy, _dz;
};
// The same scalars in the kernel's arithmetic type.  They are converted on
// the host: on GB300 a double->float conversion runs on the FP64 pipe, and
// seven of them per thread made the FP32 iteration FP64-bound.
template <typename T>
struct DyrelScalT {
    T h1, h2, dtau, cX, _dx, _dy, _dz;
    DyrelScalT() = default;
    explicit DyrelScalT(const DyrelScal& s)
        : h1((T)s.h1), h2((T)s.h2), dtau((T)s.dtau), cX((T)s.cX), _dx((T)s._dx), _dy((T)s._dy), _dz((T)s._dz) {}
};

template <typename T>
struct BC6 {
    int dir[6];  // 1 = Dirichlet, 0 = Neumann
    T val2[6];   // 2*value
};

template <typename T>
__device__ __forceinline__ T ghost(const BC6<T>& bc, int f, T inner) {
    return bc.dir[f] ? bc.val2[f] - inner : inner;
}

enum { MODE_PLAIN = 0, MODE_STOREF = 1, MODE_CHECK = 2 };

constexpr int TX = 32, TY = 8;

template <typename T, int MODE>
__global__ void __launch_bounds__(TX* TY) k_dyrel_iter(const T* __restrict__ Xin, T* __restrict__ Xout,
                                                       const T* __restrict__ R, const T* __restrict__ kx,
                                                       const T* __restrict__ ky, const T* __restrict__ kz,
                                                       const T* __restrict__ PCx, T* __restrict__ F0,
                                                       T* __restrict__ F, DyrelScalT<T> s, BC6<T> bc, int nx, int ny,
                                                       int nz, int zchunk, double* __restrict__ partials) {
    const int i = blockIdx.x * TX + threadIdx.x;
    const int j = blockIdx.y * TY + threadIdx.y;
    const int k0 = blockIdx.z * zchunk;
    const int k1 = min(nz, k0 + zchunk);
    const T h1 = s.h1, h2 = s.h2, dtau = s.dtau, cX = s.cX, _dx = s._dx, _dy = s._dy, _dz = s._dz;
    if (i < nx && j < ny && k0 < k1) {
        const int n1 = nx + 2, n2 = ny + 2;
        const long long pl = (long long)n1 * n2;  // ex plane
        const long long cpl = (long long)nx * ny;  // cell plane
        // pointers to this column
        const T* xcol = Xin + (i + 1) + (long long)n1 * (j + 1);
        T* ocol = Xout + (i + 1) + (long long)n1 * (j + 1);
        const long long ccol = i + (long long)nx * j;
        const T* kxcol = kx + i + (long long)(nx + 1) * j;
        const T* kycol = ky + i + (long long)nx * j;
        const T* kzcol = kz + ccol;
        T xc = xcol[pl * (k0 + 1)];
        T xb = (k0 == 0) ? ghost(bc, 4, xc) : xcol[pl * k0];
        T qB = -kzcol[cpl * k0] * (_dz * (xc - xb));
        for (int k = k0; k < k1; ++k) {
            const long long e = pl * (k + 1);
            const T xf = (k == nz - 1) ? ghost(bc, 5, xc) : xcol[e + pl];
            const T xw = (i == 0) ? ghost(bc, 0, xc) : xcol[e - 1];
            const T xe = (i == nx - 1) ? ghost(bc, 1, xc) : xcol[e + 1];
            const T xs = (j == 0) ? ghost(bc, 2, xc) : xcol[e - n1];
            const T xn = (j == ny - 1) ? ghost(bc, 3, xc) : xcol[e + n1];
            const long long c = ccol + cpl * k;
            const T qF = -kzcol[cpl * (k + 1)] * (_dz * (xf - xc));
            const long long fxo = (long long)(nx + 1) * ny * k;
            const long long fyo = (long long)nx * (ny + 1) * k;
            const T qW = -kxcol[fxo] * (_dx * (xc - xw));
            const T qE = -kxcol[fxo + 1] * (_dx * (xe - xc));
            const T qS = -kycol[fyo] * (_dy * (xc - xs));
            const T qN = -kycol[fyo + nx] * (_dy * (xn - xc));
            const T fu = R[c] + cX * xc + _dx * (qE - qW) + _dy * (qN - qS) + _dz * (qF - qB);
            // FP64: the reference's F /= PC (exact rounding); FP32: PCx holds 1/PC
            T f;
            if constexpr (std::is_same<T, double>::value) f = fu / PCx[c];
            else f = fu * PCx[c];
            const T f0 = h1 * F0[c] + h2 * f;
            F0[c] = f0;
            ocol[e] = xc - dtau * f0;
            if (MODE == MODE_CHECK) {  // per-cell terms of the check sums (canonical tree order)
                const T fit = F[c];
                const T d = dtau * f0;
                partials[c] = fabs((double)(f * PCx[c]));
                partials[c + cpl * nz] = (double)(-d * (f - fit));
                partials[c + 2 * cpl * nz] = (double)(d * d);
            }
            if (MODE >= MODE_STOREF) F[c] = f;
            // face ghosts of the output = BC of the input (reference state)
            if (i == 0) ocol[e - 1] = xw;
            if (i == nx - 1) ocol[e + 1] = xe;
            if (j == 0) ocol[e - n1] = xs;
            if (j == ny - 1) ocol[e + n1] = xn;
            if (k == 0) ocol[e - pl] = xb;
            if (k == nz - 1) ocol[e + pl] = xf;
            xb = xc;
            xc = xf;
            qB = qF;
        }
    }
}

// One thread per cell: the same arithmetic as k_dyrel_iter, with every load
// of a cell independent of the others (maximal memory-level parallelism, no
// per-thread z loop).  Block 32x4x2.
constexpr int CX_ = 32, CY_ = 4, CZ_ = 2;

template <typename T, int MODE>
__global__ void __launch_bounds__(CX_* CY_* CZ_) k_dyrel_cell(const T* __restrict__ Xin, T* __restrict__ Xout,
                                                             const T* __restrict__ R, const T* __restrict__ kx,
                                                             const T* __restrict__ ky, const T* __restrict__ kz,
                                                             const T* __restrict__ PCx, T* __restrict__ F0,
                                                             T* __restrict__ F, DyrelScalT<T> s, BC6<T> bc, int nx, int ny,
                                                             int nz, double* __restrict__ partials) {
    const int i = blockIdx.x * CX_ + threadIdx.x;
    const int j = blockIdx.y * CY_ + threadIdx.y;
    const int k = blockIdx.z * CZ_ + threadIdx.z;
    const T h1 = s.h1, h2 = s.h2, dtau = s.dtau, cX = s.cX, _dx = s._dx, _dy = s._dy, _dz = s._dz;
    if (i < nx && j < ny && k < nz) {
        const int n1 = nx + 2, n2 = ny + 2;
        const int pl = n1 * n2;
        const int e = (i + 1) + n1 * ((j + 1) + n2 * (k + 1));
        const int c = i + nx * (j + ny * k);
        const int fx = i + (nx + 1) * (j + ny * k);
        const int fy = i + nx * (j + (ny + 1) * k);
        const T xc = Xin[e];
        const T xw = (i == 0) ? ghost(bc, 0, xc) : Xin[e - 1];
        const T xe = (i == nx - 1) ? ghost(bc, 1, xc) : Xin[e + 1];
        const T xs = (j == 0) ? ghost(bc, 2, xc) : Xin[e - n1];
        const T xn = (j == ny - 1) ? ghost(bc, 3, xc) : Xin[e + n1];
        const T xb = (k == 0) ? ghost(bc, 4, xc) : Xin[e - pl];
        const T xf = (k == nz - 1) ? ghost(bc, 5, xc) : Xin[e + pl];
        const T qW = -kx[fx] * (_dx * (xc - xw));
        const T qE = -kx[fx + 1] * (_dx * (xe - xc));
        const T qS = -ky[fy] * (_dy * (xc - xs));
        const T qN = -ky[fy + nx] * (_dy * (xn - xc));
        const T qB = -kz[c] * (_dz * (xc - xb));
        const T qF = -kz[c + nx * ny] * (_dz * (xf - xc));
        const T fu = R[c] + cX * xc + _dx * (qE - qW) + _dy * (qN - qS) + _dz * (qF - qB);
        T f;
        if constexpr (std::is_same<T, double>::value) f = fu / PCx[c];
        else f = fu * PCx[c];
        const T f0 = h1 * F0[c] + h2 * f;
        F0[c] = f0;
        Xout[e] = xc - dtau * f0;
        if (MODE == MODE_CHECK) {  // per-cell terms of the check sums (canonical tree order)
            const T fit = F[c];
            const T d = dtau * f0;
            const int n = nx * ny * nz;
            partials[c] = fabs((double)(f * PCx[c]));
            partials[c + n] = (double)(-d * (f - fit));
            partials[c + 2 * n] = (double)(d * d);
        }
        if (MODE >= MODE_STOREF) F[c] = f;
        if (i == 0) Xout[e - 1] = xw;
        if (i == nx - 1) Xout[e + 1] = xe;
        if (j == 0) Xout[e - n1] = xs;
        if (j == ny - 1) Xout[e + n1] = xn;
        if (k == 0) Xout[e - pl] = xb;
        if (k == nz - 1) Xout[e + pl] = xf;
    }
}

// Gershgorin bound of the preconditioned operator (GershgorinPoisson!,
// Dimensional/kernels_HT3D_dimensional.jl:207-221 with a scalar rhoC) ->
// invPC = 1/D and per-block max of G/D.
template <int INV>
__global__ void k_dyrel_setup(const double* __restrict__ kx, const double* __restrict__ ky,
                              const double* __restrict__ kz, double rhoC, double transient, double dt, double dx,
                              double dy, double dz, int nx, int ny, int nz, double* __restrict__ invPC,
                              double* __restrict__ partials) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    double v[1] = {-INFINITY};
    if (i < nx && j < ny && k < nz) {
        const double kW = kx[ix3(i, j, k, nx + 1, ny)], kE = kx[ix3(i + 1, j, k, nx + 1, ny)];
        const double kS = ky[ix3(i, j, k, nx, ny + 1)], kN = ky[ix3(i, j + 1, k, nx, ny + 1)];
        const double kB = kz[ix3(i, j, k, nx, ny)], kF = kz[ix3(i, j, k + 1, nx, ny)];
        const double diag = ((kB / dz + kF / dz) / dz + (kN / dy + kS / dy) / dy + (kE / dx + kW / dx) / dx + rhoC * transient / dt);
        double g = fabs(kE / (dx * dx)) + fabs(kW / (dx * dx)) + fabs(kN / (dy * dy)) + fabs(kS / (dy * dy)) +
                   fabs(kB / (dz * dz)) + fabs(kF / (dz * dz)) + fabs(diag);
        g /= diag;
        invPC[ix3(i, j, k, nx, ny)] = INV ? 1.0 / diag : diag;
        v[0] = g;
    }
    block_reduce<RED_MAX, 1>(v);
    if (threadIdx.x == 0 && threadIdx.y == 0)
        partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = v[0];
}

// The same bound for the mixed form, with reciprocal multiplications instead
// of the reference's thirteen divisions (GB300's FP64 divide is slow; the mixed
// form does not reproduce the FP64 form's rounding): diag = sum k/dx^2 + cdiag,
// invPC = 1/diag and the per-block max of G/diag.
__global__ void k_dyrel_setup_fast(const double* __restrict__ kx, const double* __restrict__ ky,
                                   const double* __restrict__ kz, double cdiag, double _dx2, double _dy2, double _dz2,
                                   int nx, int ny, int nz, double* __restrict__ invPC, double* __restrict__ partials) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    double v[1] = {-INFINITY};
    if (i < nx && j < ny && k < nz) {
        const double kW = kx[ix3(i, j, k, nx + 1, ny)], kE = kx[ix3(i + 1, j, k, nx + 1, ny)];
        const double kS = ky[ix3(i, j, k, nx, ny + 1)], kN = ky[ix3(i, j + 1, k, nx, ny + 1)];
        const double kB = kz[ix3(i, j, k, nx, ny)], kF = kz[ix3(i, j, k + 1, nx, ny)];
        const double diag = (kB + kF) * _dz2 + (kN + kS) * _dy2 + (kE + kW) * _dx2 + cdiag;
        const double g = (fabs(kE) + fabs(kW)) * _dx2 + (fabs(kN) + fabs(kS)) * _dy2 + (fabs(kB) + fabs(kF)) * _dz2 +
                         fabs(diag);
        const double inv = 1.0 / diag;
        invPC[ix3(i, j, k, nx, ny)] = inv;
        v[0] = g * inv;
    }
    block_reduce<RED_MAX, 1>(v);
    if (threadIdx.x == 0 && threadIdx.y == 0)
        partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = v[0];
}

// copy inner cells + face ghosts (not edges/corners) of a ghosted field
template <typename T>
__global__ void k_copy_ex_faces(T* __restrict__ dst, const T* __restrict__ src, int nx, int ny, int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int n1 = nx + 2, n2 = ny + 2, n3 = nz + 2;
    if (i >= n1 || j >= n2 || k >= n3) return;
    const int nb = (i == 0 || i == n1 - 1) + (j == 0 || j == n2 - 1) + (k == 0 || k == n3 - 1);
    if (nb <= 1) dst[ix3(i, j, k, n1, n2)] = src[ix3(i, j, k, n1, n2)];
}


// One level of the canonical tree sum: block g (1024 threads) reduces
// elements [1024 g, 1024 g + 1024) of NV arrays (SPLIT: NV separate arrays
// `split` apart; otherwise NV-interleaved) with the warp-shuffle tree of
// block_reduce, padding with zeros.  The oracle's tree_sum emulates this
// order exactly.
template <int NV, bool SPLIT>
__global__ void __launch_bounds__(1024) k_tree_pass(const double* __restrict__ in, long long n, long long split,
                                                    double* __restrict__ out) {
    double v[NV];
    const long long t = (long long)blockIdx.x * 1024 + threadIdx.x;
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = t < n ? (SPLIT ? in[q * split + t] : in[t * NV + q]) : 0.0;
    block_reduce<RED_SUM, NV>(v);
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) out[(long long)blockIdx.x * NV + q] = v[q];
}

struct IterLaunch {
    int variant;  // HT3D_DYREL_ZMARCH or HT3D_DYREL_CELL
    dim3 grid, block;
    int zchunk;
    long long nblocks;
};

// elem_bytes selects the default layout when the context leaves it open
// (measured on GB300 at 255^3: FP64 is FP64-ALU bound and prefers the z-march
// tiles, FP32 is latency bound and prefers one thread per cell)
inline IterLaunch iter_launch(ht3d_ctx* ctx, int nx, int ny, int nz, int force_variant = 0, int elem_bytes = 8) {
    IterLaunch L;
    const int v = force_variant ? force_variant
                                : (ctx->dyrel_variant ? ctx->dyrel_variant
                                                      : (elem_bytes == 8 ? HT3D_DYREL_ZMARCH : HT3D_DYREL_CELL));
    L.variant = v == HT3D_DYREL_ZMARCH ? HT3D_DYREL_ZMARCH : HT3D_DYREL_CELL;
    if (L.variant == HT3D_DYREL_CELL) {
        L.block = dim3(CX_, CY_, CZ_);
        L.grid = dim3((nx + CX_ - 1) / CX_, (ny + CY_ - 1) / CY_, (nz + CZ_ - 1) / CZ_);
        L.zchunk = 1;
        L.nblocks = (long long)L.grid.x * L.grid.y * L.grid.z;
        return L;
    }
    L.block = dim3(TX, TY, 1);
    const int gx = (nx + TX - 1) / TX, gy = (ny + TY - 1) / TY;
    const long long tiles = (long long)gx * gy;
    const long long target = (long long)ctx->num_sms * 6;
    int zc = (int)std::max<long long>(1, std::min<long long>(nz, (target + tiles - 1) / tiles));
    L.zchunk = (nz + zc - 1) / zc;
    zc = (nz + L.zchunk - 1) / L.zchunk;
    L.grid = dim3(gx, gy, zc);
    L.nblocks = tiles * zc;
    return L;
}

template <typename T, int MODE>
inline void launch_iter(ht3d_ctx* ctx, const IterLaunch& L, const T* Xin, T* Xout, const T* R, const T* kx,
                        const T* ky, const T* kz, const T* PCx, T* F0, T* F, const DyrelScal& sc, const BC6<T>& bc,
                        int nx, int ny, int nz, double* partials) {
    const DyrelScalT<T> st(sc);
    if (L.variant == HT3D_DYREL_CELL)
        HT3D_LAUNCH(ctx, (k_dyrel_cell<T, MODE>), L.grid, L.block, 0, Xin, Xout, R, kx, ky, kz, PCx, F0, F, st, bc, nx,
                    ny, nz, partials);
    else
        HT3D_LAUNCH(ctx, (k_dyrel_iter<T, MODE>), L.grid, L.block, 0, Xin, Xout, R, kx, ky, kz, PCx, F0, F, st, bc, nx,
                    ny, nz, L.zchunk, partials);
}

}  // namespace


struct DyrelState {
    double lmax, lmin, dtau, c, h1, h2;
};

inline void dyrel_init_params(const ht3d_dyrel_params* prm, double lmax, DyrelState& S) {
    S.lmax = lmax;
    S.lmin = lmax / prm->lmin_ratio;
    S.dtau = 2.0 / sqrt(lmax) * prm->cfl;
    S.c = 2.0 * sqrt(S.lmin) * prm->cfact;
    S.h1 = (2 - S.c * S.dtau) / (2 + S.c * S.dtau);
    S.h2 = 2 * S.dtau / (2 + S.c * S.dtau);
}

inline bool is_check(int iter, int nitout) { return (iter % nitout == 0) || iter <= 2; }

// Host bookkeeping of a DYREL solve's check iterations
// (Dimensional/HydroThermal3D_v18.jl:457-476): the residual norm
// mean|F|/sqrt(N), the NaN and divergence errors, the Rayleigh-quotient
// update of lambda_min and the damping parameters, and the stop test.  One
// copy for every solver so they all round alike.
struct DyrelCheck {
    double nF_abs = 0.0, nF_rel = 0.0, nF_ini = 0.0;
    int checks = 0, converged = 0, status = HT3D_OK;

    // s_abs = sum |F*PC|, s_num / s_den the Rayleigh-quotient sums; returns
    // true when the solve stops at this check (error or converged).
    bool update(DyrelState& S, const ht3d_dyrel_params* prm, double s_abs, double s_num, double s_den, double ncells,
                int iter, bool stop_test) {
        ++checks;
        nF_abs = s_abs / ncells / sqrt(ncells) * prm->norm_scale;
        if (iter == 1) nF_ini = nF_abs;
        nF_rel = nF_abs / nF_ini;
        if (std::isnan(nF_abs)) {
            status = HT3D_ERR_NAN;
            return true;
        }
        if (nF_rel > 100) {
            status = HT3D_ERR_DIVERGED;
            return true;
        }
        if (iter > 1) {
            S.lmin = fabs(s_num) / fabs(s_den);
            S.c = 2.0 * sqrt(S.lmin) * prm->cfact;
            S.h1 = (2 - S.c * S.dtau) / (2 + S.c * S.dtau);
            S.h2 = 2 * S.dtau / (2 + S.c * S.dtau);
        }
        if (stop_test && (nF_abs < prm->tol_abs || nF_rel < prm->tol_rel)) {
            converged = 1;
            return true;
        }
        return false;
    }

    void fill(ht3d_dyrel_stats* st, const DyrelState& S, int iters) const {
        if (!st) return;
        st->iters = iters; st->converged = converged; st->status = status; st->checks = checks;
        st->nF_abs = nF_abs; st->nF_rel = nF_rel; st->nF_ini = nF_ini; st->lambda_min = S.lmin;
        st->lambda_max = S.lmax; st->h1 = S.h1; st->h2 = S.h2; st->dtau = S.dtau;
    }
};


// ---------------------------------------------------------------------------
// n_iter plain pseudo-iterations with fixed (h1, h2, dtau): the solver's inner
// loop without checks.  PCx is PC (FP64) or 1/PC (FP32).
// ---------------------------------------------------------------------------
template <typename T>
static int dyrel_iterate_impl(ht3d_ctx* ctx, T* X, const T* R, const T* kx, const T* ky, const T* kz, const T* PCx,
                              T* F0, double cX, double dx, double dy, double dz, const int* bc_type6,
                              const double* bc_val6, double h1, double h2, double dtau, int n_iter, int nx, int ny,
                              int nz, int slot) {
    ht3d_check_dims(nx, ny, nz, 1);
    HT3D_REQUIRE(X && R && kx && ky && kz && PCx && F0 && bc_type6 && bc_val6, "null argument");
    HT3D_REQUIRE(n_iter >= 0, "n_iter must be >= 0");
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    T* X2 = (T*)ht3d_scratch(ctx, slot, sizeof(T) * nex);
    BC6<T> bc;
    for (int f = 0; f < 6; ++f) {
        HT3D_REQUIRE(bc_type6[f] == HT3D_BC_NEUMANN || bc_type6[f] == HT3D_BC_DIRICHLET, "face BC type must be 0 or 1");
        bc.dir[f] = bc_type6[f];
        bc.val2[f] = (T)(2.0 * bc_val6[f]);
    }
    IterLaunch L = iter_launch(ctx, nx, ny, nz, 0, (int)sizeof(T));
    DyrelScal sc{h1, h2, dtau, cX, 1.0 / dx, 1.0 / dy, 1.0 / dz};
    T* cur = X;
    T* nxt = X2;
    for (int it = 0; it < n_iter; ++it) {
        launch_iter<T, MODE_PLAIN>(ctx, L, cur, nxt, R, kx, ky, kz, PCx, F0, (T*)nullptr, sc, bc, nx, ny, nz,
                                   (double*)nullptr);
        std::swap(cur, nxt);
    }
    if (cur != X) {
        dim3 b(32, 8, 1), g((nx + 2 + 31) / 32, (ny + 2 + 7) / 8, nz + 2);
        HT3D_LAUNCH(ctx, k_copy_ex_faces<T>, g, b, 0, X, cur, nx, ny, nz);
    }
    return HT3D_OK;
}


// Canonical tree sums of three n-element arrays stored back to back at
// `terms`; results land in the pinned host buffer (h_result[0..2]).
inline void tree_sum3(ht3d_ctx* ctx, const double* terms, long long n, double* work) {
    long long m = (n + 1023) / 1024;
    double* a = work;
    double* b = work + 3 * m;
    HT3D_LAUNCH(ctx, (k_tree_pass<3, true>), (unsigned)m, 1024, 0, terms, n, n, a);
    while (m > 1) {
        const long long m2 = (m + 1023) / 1024;
        HT3D_LAUNCH(ctx, (k_tree_pass<3, false>), (unsigned)m2, 1024, 0, a, m, 0LL, b);
        std::swap(a, b);
        m = m2;
    }
    ht3d_fetch_results(ctx, a, 3);
}
