// Mixed-precision DYREL solver (FP32 inner iterations, FP64 defect correction).
#include "dyrel_common.cuh"

// ---------------------------------------------------------------------------
// Mixed-precision DYREL.
//
// The FP64 solution X (caller buffer) is only touched at check iterations.
// Between checks the iteration runs in FP32 on a correction field D with
// homogeneous boundary conditions:
//     F = (Rin + cX*D + div q(D)) / diag,  F0 = h1 F0 + h2 F,  D -= dtau F0
// where Rin is the FP64 residual of X rounded to FP32 and diag the Jacobi
// diagonal PC.  At every check
// iteration of the reference schedule (iter % nitout == 0 || iter <= 2) one
// FP64 kernel folds D into X, recomputes the true FP64 residual
// (defect correction), evaluates the norms and Rayleigh-quotient sums in FP64,
// performs that iteration's update into D, and refreshes Rin.  The DYREL
// momentum F0 is stored in FP32 and carried across checks, so the iteration
// follows the FP64 one up to FP32 rounding within a check window while the
// stop test always sees the FP64 residual.
// ---------------------------------------------------------------------------
namespace {

// ---------------------------------------------------------------------------
// Padded FP32 layout of the mixed solver's inner fields.
//
// Element (i, j, k) of every FP32 field (correction D, FP32 residual Rin,
// momentum F0, F, face conductivities) sits at i + PX*(j + PY*k) with
// PX = nx+1 rounded up to 32 (128-byte rows), PY = ny+1 and nz+1 planes.  One
// index therefore addresses a cell, its west x-face, its south y-face and its
// bottom z-face; the east/north/front faces are +1, +PX, +PX*PY.  There is no
// ghost storage: ghosts are evaluated from the BCs.  Padding stays zero.
// ---------------------------------------------------------------------------
struct Pad {
    int nx, ny, nz, PX, PY, nq;  // nq: 4-cell quads per row
    long long plane, size;
};
inline Pad make_pad(int nx, int ny, int nz) {
    Pad p;
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.PX = ((nx + 1 + 31) / 32) * 32;
    p.PY = ny + 1;
    p.nq = (nx + 3) / 4;
    p.plane = (long long)p.PX * p.PY;
    p.size = p.plane * (nz + 1);
    return p;
}

// reference column-major array of ax x ay x az -> padded FP32
__global__ void k_pack(float* __restrict__ dst, const double* __restrict__ src, int ax, int ay, int az, Pad p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= ax || j >= ay || k >= az) return;
    dst[i + (long long)p.PX * j + p.plane * k] = (float)src[i + (long long)ax * (j + (long long)ay * k)];
}
// padded FP32 cell field -> reference cell array (FP64)
__global__ void k_unpack(double* __restrict__ dst, const float* __restrict__ src, Pad p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= p.nx || j >= p.ny || k >= p.nz) return;
    dst[i + (long long)p.nx * (j + (long long)p.ny * k)] = (double)src[i + (long long)p.PX * j + p.plane * k];
}

__device__ __forceinline__ float c4(const float4& v, int m) {
    return m == 0 ? v.x : (m == 1 ? v.y : (m == 2 ? v.z : v.w));
}

// FP32 inner iteration of the mixed solver on the padded layout.  Thread t
// of plane k owns quad q = t % nq (cells 4q..4q+3) of row j = t / nq and
// moves every field with 16-byte loads; the x-neighbours across the quad
// edges come from the adjacent lanes (same row) by warp shuffles, or from a
// scalar load at a warp edge.  The Jacobi diagonal (the Gershgorin D of the
// operator, sum of k/dx^2 over the six faces + cX) is recomputed from the
// face conductivities already in registers instead of being streamed.
//     F = (Rin + cX D + div q(D)) / diag ;  F0 = h1 F0 + h2 F ;  D -= dtau F0
template <bool STOREF>
__global__ void __launch_bounds__(256) k_mixed_inner(const float* __restrict__ Din, float* __restrict__ Dout,
                                                     const float* __restrict__ Rin, const float* __restrict__ kx,
                                                     const float* __restrict__ ky, const float* __restrict__ kz,
                                                     float* __restrict__ F0, float* __restrict__ F,
                                                     DyrelScalT<float> s, BC6<float> bc, Pad p) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int q = t % p.nq;
    int j = t / p.nq;
    const bool act = j < p.ny;
    if (!act) j = p.ny - 1;  // stays in the shuffles, loads in-bounds data, stores nothing
    const int i0 = 4 * q;
    const long long base = i0 + (long long)p.PX * j + p.plane * k;
    const float4 d = *reinterpret_cast<const float4*>(Din + base);
    const float4 kx4 = *reinterpret_cast<const float4*>(kx + base);
    // every lane takes part in the shuffles
    const float dW_sh = __shfl_up_sync(0xffffffffu, d.w, 1);
    const float dE_sh = __shfl_down_sync(0xffffffffu, d.x, 1);
    const float kE_sh = __shfl_down_sync(0xffffffffu, kx4.x, 1);
    const bool south = j > 0, north = j < p.ny - 1, back = k > 0, front = k < p.nz - 1;
    const float4 dS = south ? *reinterpret_cast<const float4*>(Din + base - p.PX) : d;
    const float4 dN = north ? *reinterpret_cast<const float4*>(Din + base + p.PX) : d;
    const float4 dB = back ? *reinterpret_cast<const float4*>(Din + base - p.plane) : d;
    const float4 dF = front ? *reinterpret_cast<const float4*>(Din + base + p.plane) : d;
    const float4 kyS = *reinterpret_cast<const float4*>(ky + base);
    const float4 kyN = *reinterpret_cast<const float4*>(ky + base + p.PX);
    const float4 kzB = *reinterpret_cast<const float4*>(kz + base);
    const float4 kzF = *reinterpret_cast<const float4*>(kz + base + p.plane);
    const float4 r4 = *reinterpret_cast<const float4*>(Rin + base);
    const float4 f04 = *reinterpret_cast<const float4*>(F0 + base);
    // west neighbour of cell i0, east neighbour of cell i0+3, east face of cell i0+3
    float dW = 0.f, dE = 0.f, kE3 = 0.f;
    if (i0 > 0) dW = lane > 0 ? dW_sh : Din[base - 1];
    if (i0 + 4 < p.nx) dE = lane < 31 ? dE_sh : Din[base + 4];
    if (i0 + 3 < p.nx) kE3 = (lane < 31 && q < p.nq - 1) ? kE_sh : kx[base + 4];
    const float h1 = s.h1, h2 = s.h2, dtau = s.dtau, cX = s.cX, _dx = s._dx, _dy = s._dy, _dz = s._dz;
    const float _dx2 = _dx * _dx, _dy2 = _dy * _dy, _dz2 = _dz * _dz;
    float outD[4], outF0[4], outF[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int i = i0 + m;
        const float xc = c4(d, m);
        const float xw = (i == 0) ? ghost(bc, 0, xc) : (m == 0 ? dW : c4(d, m - 1));
        const float xe = (i == p.nx - 1) ? ghost(bc, 1, xc) : (m == 3 ? dE : c4(d, m + 1));
        const float xs = south ? c4(dS, m) : ghost(bc, 2, xc);
        const float xn = north ? c4(dN, m) : ghost(bc, 3, xc);
        const float xb = back ? c4(dB, m) : ghost(bc, 4, xc);
        const float xf = front ? c4(dF, m) : ghost(bc, 5, xc);
        const float kW = c4(kx4, m), kE = m == 3 ? kE3 : c4(kx4, m + 1);
        const float kS = c4(kyS, m), kN = c4(kyN, m), kB = c4(kzB, m), kF = c4(kzF, m);
        const float qW = -kW * (_dx * (xc - xw));
        const float qE = -kE * (_dx * (xe - xc));
        const float qS = -kS * (_dy * (xc - xs));
        const float qN = -kN * (_dy * (xn - xc));
        const float qB = -kB * (_dz * (xc - xb));
        const float qF = -kF * (_dz * (xf - xc));
        const float fu = c4(r4, m) + cX * xc + _dx * (qE - qW) + _dy * (qN - qS) + _dz * (qF - qB);
        const float diag = (kW + kE) * _dx2 + (kS + kN) * _dy2 + (kB + kF) * _dz2 + cX;
        const float f = __fdividef(fu, diag);
        const float f0 = h1 * c4(f04, m) + h2 * f;
        const bool valid = i < p.nx;
        outF0[m] = valid ? f0 : 0.f;
        outD[m] = valid ? xc - dtau * f0 : 0.f;
        outF[m] = valid ? f : 0.f;
    }
    if (!act) return;
    *reinterpret_cast<float4*>(F0 + base) = make_float4(outF0[0], outF0[1], outF0[2], outF0[3]);
    *reinterpret_cast<float4*>(Dout + base) = make_float4(outD[0], outD[1], outD[2], outD[3]);
    if (STOREF) *reinterpret_cast<float4*>(F + base) = make_float4(outF[0], outF[1], outF[2], outF[3]);
}

// FP64 check iteration of the mixed solver (see above).  FP64 fields in the
// reference layout, FP32 fields in the padded layout.
__global__ void __launch_bounds__(TX* TY) k_mixed_check(
    const double* __restrict__ Xin, double* __restrict__ Xout, const float* __restrict__ Din, float* __restrict__ Dout,
    const double* __restrict__ R, const double* __restrict__ kx, const double* __restrict__ ky,
    const double* __restrict__ kz, const double* __restrict__ invPC, float* __restrict__ F0,
    float* __restrict__ F32, double* __restrict__ F64, float* __restrict__ Rin, DyrelScal s, BC6<double> bc,
    Pad p, int zchunk, double* __restrict__ partials) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int i = blockIdx.x * TX + threadIdx.x;
    const int j = blockIdx.y * TY + threadIdx.y;
    const int k0 = blockIdx.z * zchunk;
    const int k1 = min(nz, k0 + zchunk);
    double acc[3] = {0.0, 0.0, 0.0};
    if (i < nx && j < ny && k0 < k1) {
        const int n1 = nx + 2, n2 = ny + 2;
        const long long pl = (long long)n1 * n2, cpl = (long long)nx * ny, pp = p.plane;
        const long long col = (i + 1) + (long long)n1 * (j + 1);
        const long long pcol = i + (long long)p.PX * j;
        const double* xcol = Xin + col;
        const float* dcol = Din + pcol;
        double* ocol = Xout + col;
        const long long ccol = i + (long long)nx * j;
        const double* kxcol = kx + i + (long long)(nx + 1) * j;
        const double* kycol = ky + i + (long long)nx * j;
        const double* kzcol = kz + ccol;
        auto fold = [&](long long e, long long pe) { return xcol[e] + (double)dcol[pe]; };
        double xc = fold(pl * (k0 + 1), pp * k0);
        double xb = (k0 == 0) ? ghost(bc, 4, xc) : fold(pl * k0, pp * (k0 - 1));
        double qB = -kzcol[cpl * k0] * (s._dz * (xc - xb));
        for (int k = k0; k < k1; ++k) {
            const long long e = pl * (k + 1), pe = pp * k;
            const double xf = (k == nz - 1) ? ghost(bc, 5, xc) : fold(e + pl, pe + pp);
            const double xw = (i == 0) ? ghost(bc, 0, xc) : fold(e - 1, pe - 1);
            const double xe = (i == nx - 1) ? ghost(bc, 1, xc) : fold(e + 1, pe + 1);
            const double xs = (j == 0) ? ghost(bc, 2, xc) : fold(e - n1, pe - p.PX);
            const double xn = (j == ny - 1) ? ghost(bc, 3, xc) : fold(e + n1, pe + p.PX);
            const long long c = ccol + cpl * k, pc = pcol + pe;
            const double qF = -kzcol[cpl * (k + 1)] * (s._dz * (xf - xc));
            const long long fxo = (long long)(nx + 1) * ny * k, fyo = (long long)nx * (ny + 1) * k;
            const double qW = -kxcol[fxo] * (s._dx * (xc - xw));
            const double qE = -kxcol[fxo + 1] * (s._dx * (xe - xc));
            const double qS = -kycol[fyo] * (s._dy * (xc - xs));
            const double qN = -kycol[fyo + nx] * (s._dy * (xn - xc));
            const double fu = R[c] + s.cX * xc + s._dx * (qE - qW) + s._dy * (qN - qS) + s._dz * (qF - qB);
            const double f = fu * invPC[c];
            const double f0 = s.h1 * (double)F0[pc] + s.h2 * f;
            const double fit = (double)F32[pc];
            const double d = s.dtau * f0;
            acc[0] += fabs(fu);
            acc[1] += -d * (f - fit);
            acc[2] += d * d;
            F0[pc] = (float)f0;
            F32[pc] = (float)f;
            F64[c] = f;
            Rin[pc] = (float)fu;
            Dout[pc] = (float)(-d);
            ocol[e] = xc;
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
    block_reduce<RED_SUM, 3>(acc);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const long long b = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
        partials[3 * b + 0] = acc[0];
        partials[3 * b + 1] = acc[1];
        partials[3 * b + 2] = acc[2];
    }
}

// Final fold X = X + D of the inner cells.  The face ghosts receive the BC
// of the state before the last pseudo-iteration, as the reference leaves
// them: X + Dprev when the last iteration was an inner one (Dprev is the
// other ping-pong buffer); when it ran the FP64 kernel (Dprev == nullptr)
// that kernel has already written them.
__global__ void k_mixed_fold(double* __restrict__ X, const float* __restrict__ D, const float* __restrict__ Dprev,
                             BC6<double> bc, Pad p) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= nx || j >= ny || k >= nz) return;
    const int n1 = nx + 2, n2 = ny + 2;
    const long long pl = (long long)n1 * n2;
    const long long e = (i + 1) + (long long)n1 * (j + 1) + pl * (k + 1);
    const long long pe = i + (long long)p.PX * j + p.plane * k;
    const double x0 = X[e];
    X[e] = x0 + (double)D[pe];
    if (!Dprev) return;
    const double x = x0 + (double)Dprev[pe];
    if (i == 0) X[e - 1] = ghost(bc, 0, x);
    if (i == nx - 1) X[e + 1] = ghost(bc, 1, x);
    if (j == 0) X[e - n1] = ghost(bc, 2, x);
    if (j == ny - 1) X[e + n1] = ghost(bc, 3, x);
    if (k == 0) X[e - pl] = ghost(bc, 4, x);
    if (k == nz - 1) X[e + pl] = ghost(bc, 5, x);
}

// Live timing of the inner-iteration runs (HT3D_TUNE_TIME_INNER): an event
// pair around every run of consecutive inner launches on the ctx stream.
struct InnerTimer {
    ht3d_ctx* ctx;
    bool on, open = false;
    int pairs = 0;
    unsigned long long launches = 0;
    explicit InnerTimer(ht3d_ctx* c) : ctx(c), on(c->time_inner != 0) {}
    void begin() {
        if (!on || open) return;
        const int need = 2 * (pairs + 1);
        while ((int)ctx->events.size() < need) {
            cudaEvent_t ev;
            HT3D_CUDA(cudaEventCreate(&ev));
            ctx->events.push_back(ev);
        }
        HT3D_CUDA(cudaEventRecord(ctx->events[2 * pairs], ctx->stream));
        open = true;
    }
    void count() { if (on) ++launches; }
    void end() {
        if (!on || !open) return;
        HT3D_CUDA(cudaEventRecord(ctx->events[2 * pairs + 1], ctx->stream));
        ++pairs;
        open = false;
    }
    void collect() {
        end();
        if (!on || pairs == 0) return;
        HT3D_CUDA(cudaEventSynchronize(ctx->events[2 * pairs - 1]));
        double ms = 0.0;
        for (int q = 0; q < pairs; ++q) {
            float e = 0.f;
            HT3D_CUDA(cudaEventElapsedTime(&e, ctx->events[2 * q], ctx->events[2 * q + 1]));
            ms += e;
        }
        ctx->inner_ms += ms;
        ctx->inner_launches += launches;
    }
};

}  // namespace

int ht3d_dyrel_solve_mixed(ht3d_ctx* ctx, double* X, const double* R, const double* kx, const double* ky,
                           const double* kz, double cX, double dx, double dy, double dz, const int* bc_type6,
                           const double* bc_val6, const ht3d_dyrel_params* prm, int n_iter_fixed, double* F,
                           double* F0, ht3d_dyrel_stats* st, int nx, int ny, int nz) {
    const long long n = (long long)nx * ny * nz;
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    const Pad P = make_pad(nx, ny, nz);
    HT3D_REQUIRE(P.size < (1LL << 31), "grid too large for the padded FP32 layout");
    const size_t pbytes = sizeof(float) * (size_t)P.size;
    double* invPC = (double*)ht3d_scratch(ctx, SLOT_PC, sizeof(double) * n);
    double* X2 = (double*)ht3d_scratch(ctx, SLOT_X2, sizeof(double) * nex);
    float* Da = (float*)ht3d_scratch(ctx, SLOT_F32_X, pbytes);
    float* Db = (float*)ht3d_scratch(ctx, SLOT_F32_X2, pbytes);
    float* F0s = (float*)ht3d_scratch(ctx, SLOT_F32_F0, pbytes);
    float* Fs = (float*)ht3d_scratch(ctx, SLOT_F32_F, pbytes);
    float* Rin = (float*)ht3d_scratch(ctx, SLOT_F32_R, pbytes);
    float* kx32 = (float*)ht3d_scratch(ctx, SLOT_F32_KX, pbytes);
    float* ky32 = (float*)ht3d_scratch(ctx, SLOT_F32_KY, pbytes);
    float* kz32 = (float*)ht3d_scratch(ctx, SLOT_F32_KZ, pbytes);
    IterLaunch LC = iter_launch(ctx, nx, ny, nz, HT3D_DYREL_ZMARCH);  // layout of the FP64 check kernel
    const long long nparts = std::max<long long>(LC.nblocks, (long long)((nx + 31) / 32) * ((ny + 7) / 8) * nz);
    double* parts = (double*)ht3d_scratch(ctx, SLOT_PARTIALS, sizeof(double) * 3 * nparts);
    double* dres = (double*)ht3d_scratch(ctx, SLOT_RESULT, sizeof(double) * 64);

    BC6<double> bc;
    BC6<float> bch;  // homogeneous (correction) BCs
    for (int f = 0; f < 6; ++f) {
        HT3D_REQUIRE(bc_type6[f] == HT3D_BC_NEUMANN || bc_type6[f] == HT3D_BC_DIRICHLET, "face BC type must be 0 or 1");
        bc.dir[f] = bch.dir[f] = bc_type6[f];
        bc.val2[f] = 2.0 * bc_val6[f];
        bch.val2[f] = 0.0f;
    }
    const dim3 b2(32, 8, 1), gc((nx + 31) / 32, (ny + 7) / 8, nz);
    {
        const double transient = cX != 0.0 ? 1.0 : 0.0, dt = cX != 0.0 ? 1.0 / cX : 1.0;
        HT3D_LAUNCH(ctx, k_dyrel_setup<1>, gc, b2, 0, kx, ky, kz, 1.0, transient, dt, dx, dy, dz, nx, ny, nz, invPC, parts);
        HT3D_LAUNCH(ctx, (k_reduce_partials<RED_MAX, 1>), 1, 1024, 0, parts, (int)(gc.x * gc.y * gc.z), dres);
    }
    for (float* a : {Da, Db, F0s, Fs, Rin, kx32, ky32, kz32}) HT3D_CUDA(cudaMemsetAsync(a, 0, pbytes, ctx->stream));
    HT3D_LAUNCH(ctx, k_pack, dim3((nx + 1 + 31) / 32, (ny + 7) / 8, nz), b2, 0, kx32, kx, nx + 1, ny, nz, P);
    HT3D_LAUNCH(ctx, k_pack, dim3((nx + 31) / 32, (ny + 1 + 7) / 8, nz), b2, 0, ky32, ky, nx, ny + 1, nz, P);
    HT3D_LAUNCH(ctx, k_pack, dim3((nx + 31) / 32, (ny + 7) / 8, nz + 1), b2, 0, kz32, kz, nx, ny, nz + 1, P);
    ht3d_fetch_results(ctx, dres, 1);
    DyrelState S;
    dyrel_init_params(prm, ctx->h_result[0], S);

    DyrelScal sc;
    sc.cX = cX;
    sc._dx = 1.0 / dx;
    sc._dy = 1.0 / dy;
    sc._dz = 1.0 / dz;
    const dim3 ib(256), ig((unsigned)(((long long)P.nq * ny + 255) / 256), (unsigned)nz);
    InnerTimer timer(ctx);
    double* xcur = X;
    double* xnxt = X2;
    float* dcur = Da;
    float* dnxt = Db;
    double nF_abs = 0., nF_rel = 0., nF_ini = 0.;
    int it_done = 0, converged = 0, status = HT3D_OK, checks = 0;
    bool last_fp64 = false;  // the last iteration ran the FP64 kernel (check or refresh)
    const int nmax = n_iter_fixed > 0 ? n_iter_fixed : prm->nitmax;
    const int refresh_every = ctx->mixed_refresh;
    for (int iter = 1; iter <= nmax; ++iter) {
        const bool chk = is_check(iter, prm->nitout);
        // defect-correction refresh between the reference's checks: fold D into X
        // and recompute the FP64 residual so the FP32 iteration never works
        // below its own precision (no stop test, no parameter update)
        const bool refresh = !chk && refresh_every > 0 && iter % refresh_every == 0;
        const bool storef = !chk && (iter == nmax || is_check(iter + 1, prm->nitout));
        sc.h1 = S.h1;
        sc.h2 = S.h2;
        sc.dtau = S.dtau;
        if (chk || refresh) {
            timer.end();
            HT3D_LAUNCH(ctx, k_mixed_check, LC.grid, LC.block, 0, xcur, xnxt, dcur, dnxt, R, kx, ky, kz, invPC, F0s, Fs,
                        F, Rin, sc, bc, P, LC.zchunk, parts);
            std::swap(xcur, xnxt);
        } else {
            const DyrelScalT<float> s32(sc);
            timer.begin();
            if (storef)
                HT3D_LAUNCH(ctx, k_mixed_inner<true>, ig, ib, 0, dcur, dnxt, Rin, kx32, ky32, kz32, F0s, Fs, s32, bch, P);
            else
                HT3D_LAUNCH(ctx, k_mixed_inner<false>, ig, ib, 0, dcur, dnxt, Rin, kx32, ky32, kz32, F0s, Fs, s32, bch, P);
            timer.count();
        }
        std::swap(dcur, dnxt);
        it_done = iter;
        last_fp64 = chk || refresh;
        if (chk) {
            ++checks;
            HT3D_LAUNCH(ctx, (k_reduce_partials<RED_SUM, 3>), 1, 1024, 0, parts, (int)LC.nblocks, dres);
            ht3d_fetch_results(ctx, dres, 3);
            const double s_abs = ctx->h_result[0], s_num = ctx->h_result[1], s_den = ctx->h_result[2];
            nF_abs = s_abs / (double)n / sqrt((double)n) * prm->norm_scale;
            if (iter == 1) nF_ini = nF_abs;
            nF_rel = nF_abs / nF_ini;
            if (std::isnan(nF_abs)) { status = HT3D_ERR_NAN; break; }
            if (nF_rel > 100) { status = HT3D_ERR_DIVERGED; break; }
            if (iter > 1) {
                S.lmin = fabs(s_num) / fabs(s_den);
                S.c = 2.0 * sqrt(S.lmin) * prm->cfact;
                S.h1 = (2 - S.c * S.dtau) / (2 + S.c * S.dtau);
                S.h2 = 2 * S.dtau / (2 + S.c * S.dtau);
            }
            if (n_iter_fixed <= 0 && (nF_abs < prm->tol_abs || nF_rel < prm->tol_rel)) { converged = 1; break; }
        }
    }
    timer.end();
    // final fold of the correction into the FP64 solution
    HT3D_LAUNCH(ctx, k_mixed_fold, gc, b2, 0, xcur, dcur, last_fp64 ? nullptr : dnxt, bc, P);
    if (xcur != X) {
        dim3 g((nx + 2 + 31) / 32, (ny + 2 + 7) / 8, nz + 2);
        HT3D_LAUNCH(ctx, k_copy_ex_faces<double>, g, b2, 0, X, xcur, nx, ny, nz);
    }
    HT3D_LAUNCH(ctx, k_unpack, gc, b2, 0, F0, F0s, P);
    if (!last_fp64) HT3D_LAUNCH(ctx, k_unpack, gc, b2, 0, F, Fs, P);
    timer.collect();
    if (st) {
        st->iters = it_done; st->converged = converged; st->status = status; st->checks = checks;
        st->nF_abs = nF_abs; st->nF_rel = nF_rel; st->nF_ini = nF_ini; st->lambda_min = S.lmin;
        st->lambda_max = S.lmax; st->h1 = S.h1; st->h2 = S.h2; st->dtau = S.dtau;
    }
    return status;
}


extern "C" int ht3d_dyrel_iterate_f32(ht3d_ctx* ctx, float* X_ex, const float* R, const float* kx, const float* ky,
                                      const float* kz, const float* invPC, float* F0, double cX, double dx, double dy,
                                      double dz, const int* bc_type6, const double* bc_val6, double h1, double h2,
                                      double dtau, int n_iter, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        return dyrel_iterate_impl<float>(ctx, X_ex, R, kx, ky, kz, invPC, F0, cX, dx, dy, dz, bc_type6, bc_val6, h1, h2,
                                         dtau, n_iter, nx, ny, nz, SLOT_AUX1);
    });
}
