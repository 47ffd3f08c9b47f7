// Mixed-precision DYREL solver (FP32 inner iterations, FP64 defect correction).
#include <cuda.h>
#include <algorithm>
#include <cstddef>
#include <mutex>

#include "dyrel_common.cuh"
#include "ensemble_internal.cuh"

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
// momentum is not stored: F0 = (Dprev - D) / dtau_prev follows from the
// correction before the last update, which the iteration streams instead of
// reading and writing F0 (seven fields per iteration instead of eight).  It is
// carried across checks (Dprev = 0 after a fold), so the iteration follows
// the FP64 one up to FP32 rounding within a check window while the stop test
// always sees the FP64 residual.
// ---------------------------------------------------------------------------
namespace {

// ---------------------------------------------------------------------------
// Padded FP32 layout of the mixed solver's inner fields.
//
// Element (i, j, k) of every FP32 field (corrections D and Dprev, FP32
// residual Rin, F, face conductivities) sits at i + PX*(j + PY*k) with
// PX = nx+1 rounded up to 8 (rows of whole 32-byte sectors, so every quad is
// 16-byte aligned and every tensor-map stride a multiple of 16 bytes; rounding
// to 32 cost the 31-95-cell ensemble members about a fifth of their bytes in
// padding), PY = ny+1 and nz+1 planes.  One
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
    p.PX = ((nx + 1 + 7) / 8) * 8;
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

// Scalars of the FP32 iterations of the mixed solver, converted on the host.
// The DYREL update F0' = h1 F0 + h2 F, x' = x - dtau F0' runs without a stored
// momentum: F0 = (xprev - x) / dtau_prev is implied by the correction before
// the last update (dtau_prev the dtau of that update), so
//     x' = x + mom (x - xprev) - dh2 F,   mom = h1 dtau / dtau_prev,  dh2 = dtau h2
// and an iteration streams the previous correction instead of reading and
// writing F0.  mom = h1 except on the first iteration after a parameter update.
struct MixScal {
    float mom, dh2;             // inner update
    float h1, h2, dtau;         // the FP64 check / refresh iteration's own update
    float dtau_prev;            // dtau of the update that produced the current correction
    float cX, _dx, _dy, _dz;
};
inline MixScal mix_scal(const DyrelScal& s, double dtau_prev) {
    MixScal m;
    m.mom = (float)(s.h1 * s.dtau / dtau_prev);
    m.dh2 = (float)(s.dtau * s.h2);
    m.h1 = (float)s.h1;
    m.h2 = (float)s.h2;
    m.dtau = (float)s.dtau;
    m.dtau_prev = (float)dtau_prev;
    m.cX = (float)s.cX;
    m._dx = (float)s._dx;
    m._dy = (float)s._dy;
    m._dz = (float)s._dz;
    return m;
}

// One cell of the FP32 inner iteration (the single place its arithmetic is
// written, so every kernel that updates a cell rounds alike):
//     F = (R + cX x + div q(x)) * (1 / diag),  x' = x + mom (x - xprev) - dh2 F
// with q = -k dx on the six faces and diag = sum of k/dx^2 over them + cX;
// div q is evaluated per axis as dx^2 (k_in (x - x_in) - k_out (x_out - x)).
// Every operation is an explicit round-to-nearest intrinsic (and 1 / diag one
// approximate reciprocal): the compiler may neither contract nor reassociate
// them, so the value of a cell does not depend on the kernel it is inlined
// into (k_mixed_inner shares fluxes between the four cells of a quad,
// k_mixed_inner2 does not and hands 1 / diag from its first iteration of a
// pass to the second).
// approximate reciprocal (one MUFU operation, ~1 ulp); the diagonals it is
// applied to are positive normal numbers
__device__ __forceinline__ float rcp_approx(float v) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}
// 1 / diag of a cell: diag = cX + sum over the faces of k/dx^2
__device__ __forceinline__ float mixed_rdiag(float kW, float kE, float kS, float kN, float kB, float kF, float cX,
                                             float _dx2, float _dy2, float _dz2) {
    float diag = __fmaf_rn(__fadd_rn(kW, kE), _dx2, cX);
    diag = __fmaf_rn(__fadd_rn(kS, kN), _dy2, diag);
    diag = __fmaf_rn(__fadd_rn(kB, kF), _dz2, diag);
    return rcp_approx(diag);
}
// the cell update given its 1 / diag
__device__ __forceinline__ void mixed_cell_rd(float xc, float xw, float xe, float xs, float xn, float xb, float xf,
                                              float kW, float kE, float kS, float kN, float kB, float kF, float r,
                                              float xprev, float rd, float mom, float dh2, float cX, float _dx2,
                                              float _dy2, float _dz2, float& f, float& xnew) {
    // dx (qE - qW) with q = -k dx (x_out - x_in) is dx^2 (kW (xc - xw) - kE (xe - xc))
    const float gx = __fmaf_rn(kW, __fsub_rn(xc, xw), -__fmul_rn(kE, __fsub_rn(xe, xc)));
    const float gy = __fmaf_rn(kS, __fsub_rn(xc, xs), -__fmul_rn(kN, __fsub_rn(xn, xc)));
    const float gz = __fmaf_rn(kB, __fsub_rn(xc, xb), -__fmul_rn(kF, __fsub_rn(xf, xc)));
    float fu = __fmaf_rn(cX, xc, r);
    fu = __fmaf_rn(_dx2, gx, fu);
    fu = __fmaf_rn(_dy2, gy, fu);
    fu = __fmaf_rn(_dz2, gz, fu);
    f = __fmul_rn(fu, rd);
    xnew = __fmaf_rn(mom, __fsub_rn(xc, xprev), __fmaf_rn(-dh2, f, xc));
}
__device__ __forceinline__ void mixed_cell(float xc, float xw, float xe, float xs, float xn, float xb, float xf,
                                           float kW, float kE, float kS, float kN, float kB, float kF, float r,
                                           float xprev, float mom, float dh2, float cX, float _dx, float _dy,
                                           float _dz, float _dx2, float _dy2, float _dz2, float& f, float& xnew) {
    const float rd = mixed_rdiag(kW, kE, kS, kN, kB, kF, cX, _dx2, _dy2, _dz2);
    mixed_cell_rd(xc, xw, xe, xs, xn, xb, xf, kW, kE, kS, kN, kB, kF, r, xprev, rd, mom, dh2, cX, _dx2, _dy2, _dz2, f,
                  xnew);
}

// Ghost value of the FP32 correction fields: their BCs are homogeneous (the
// Dirichlet value lives in the FP64 state), so a ghost is -v (Dirichlet) or v
// (Neumann): one select instead of the general 2 value - v.  Every FP32
// kernel of the mixed form uses it, so they agree bit for bit (a zero ghost
// may carry the other sign than 0 - v would).
__device__ __forceinline__ float hghost(const BC6<float>& bc, int f, float v) { return bc.dir[f] ? -v : v; }

// x-neighbours across a quad's edges: the west neighbour of cell i0, the east
// neighbour of cell i0+3 and the east face of cell i0+3, from the adjacent
// lanes (same row) by warp shuffles, or by a scalar load at a warp edge.
// Every lane of the warp takes part in the shuffles.
__device__ __forceinline__ void quad_x_edges(const float* __restrict__ Din, const float* __restrict__ kx,
                                             const float4& d, const float4& kx4, long long base, int i0, int q,
                                             const Pad& p, int lane, float& dW, float& dE, float& kE3) {
    const float dW_sh = __shfl_up_sync(0xffffffffu, d.w, 1);
    const float dE_sh = __shfl_down_sync(0xffffffffu, d.x, 1);
    const float kE_sh = __shfl_down_sync(0xffffffffu, kx4.x, 1);
    dW = 0.f;
    dE = 0.f;
    kE3 = 0.f;
    if (i0 > 0) dW = lane > 0 ? dW_sh : Din[base - 1];
    if (i0 + 4 < p.nx) dE = lane < 31 ? dE_sh : Din[base + 4];
    if (i0 + 3 < p.nx) kE3 = (lane < 31 && q < p.nq - 1) ? kE_sh : kx[base + 4];
}

// The four cells of a quad (mixed_cell each) from the loaded neighbourhood;
// stores D' (and F) unless act is false.  Neighbours beyond the grid are the
// ghost values of the BCs (dS .. dF are not read there).
template <bool STOREF>
__device__ __forceinline__ void quad_cells(const float4& d, const float4& kx4, const float4& dS, const float4& dN,
                                           const float4& dB, const float4& dF, const float4& kyS, const float4& kyN,
                                           const float4& kzB, const float4& kzF, const float4& r4, const float4& dp4,
                                           float dW, float dE, float kE3, bool south, bool north, bool back,
                                           bool front, int i0, const Pad& p, const MixScal& s, const BC6<float>& bc,
                                           float* __restrict__ Dio, float* __restrict__ F, long long base, bool act) {
    const float mom = s.mom, dh2 = s.dh2, cX = s.cX, _dx = s._dx, _dy = s._dy, _dz = s._dz;
    const float _dx2 = __fmul_rn(_dx, _dx), _dy2 = __fmul_rn(_dy, _dy), _dz2 = __fmul_rn(_dz, _dz);
    float outD[4], outF[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int i = i0 + m;
        const float xc = c4(d, m);
        const float xw = (i == 0) ? hghost(bc, 0, xc) : (m == 0 ? dW : c4(d, m - 1));
        const float xe = (i == p.nx - 1) ? hghost(bc, 1, xc) : (m == 3 ? dE : c4(d, m + 1));
        const float xs = south ? c4(dS, m) : hghost(bc, 2, xc);
        const float xn = north ? c4(dN, m) : hghost(bc, 3, xc);
        const float xb = back ? c4(dB, m) : hghost(bc, 4, xc);
        const float xf = front ? c4(dF, m) : hghost(bc, 5, xc);
        const float kW = c4(kx4, m), kE = m == 3 ? kE3 : c4(kx4, m + 1);
        const float kS = c4(kyS, m), kN = c4(kyN, m), kB = c4(kzB, m), kF = c4(kzF, m);
        float f, xn1;
        mixed_cell(xc, xw, xe, xs, xn, xb, xf, kW, kE, kS, kN, kB, kF, c4(r4, m), c4(dp4, m), mom, dh2, cX, _dx, _dy,
                   _dz, _dx2, _dy2, _dz2, f, xn1);
        outD[m] = xn1;
        outF[m] = f;
    }
    if (i0 + 4 > p.nx) {  // the row's last quad: its padding cells stay zero
#pragma unroll
        for (int m = 0; m < 4; ++m)
            if (i0 + m >= p.nx) outD[m] = outF[m] = 0.f;
    }
    if (!act) return;
    *reinterpret_cast<float4*>(Dio + base) = make_float4(outD[0], outD[1], outD[2], outD[3]);
    if (STOREF) *reinterpret_cast<float4*>(F + base) = make_float4(outF[0], outF[1], outF[2], outF[3]);
}

// FP32 inner iteration of the mixed solver on the padded layout, for the
// quad of cells 4q..4q+3 of row j, plane k (t = q + nq*j is the thread's
// position in the plane).  Every field moves with 16-byte loads; the
// x-neighbours across the quad edges come from the adjacent lanes (same
// row) by warp shuffles, or from a scalar load at a warp edge.  The Jacobi
// diagonal (the Gershgorin D of the operator, sum of k/dx^2 over the six
// faces + cX) is recomputed from the face conductivities already in
// registers instead of being streamed.
//     F = (Rin + cX D + div q(D)) / diag ;  D' = D + mom (D - Dprev) - dh2 F
// Dio holds Dprev on entry (read at the thread's own cells only, so the
// update can overwrite it in place); prev0 means Dprev = 0 (the correction
// was just folded into the FP64 solution) and skips its load.  Seven fields
// stream per iteration: D (with its neighbour rows), Dprev/D', Rin, kx, ky, kz.
// All 32 lanes of the warp must call it.  Lanes past the grid (j >= ny, or
// live == false) take part with in-bounds loads and store nothing.
template <bool STOREF>
__device__ __forceinline__ void mixed_quad(const float* __restrict__ Din, float* __restrict__ Dio,
                                           const float* __restrict__ Rin, const float* __restrict__ kx,
                                           const float* __restrict__ ky, const float* __restrict__ kz,
                                           float* __restrict__ F, const MixScal& s, bool prev0, const BC6<float>& bc,
                                           const Pad& p, int t, int k, int lane, bool live = true) {
    const int q = t % p.nq;
    int j = t / p.nq;
    const bool act = live && j < p.ny;
    if (j >= p.ny) j = p.ny - 1;
    const int i0 = 4 * q;
    const long long base = i0 + (long long)p.PX * j + p.plane * k;
    const float4 d = *reinterpret_cast<const float4*>(Din + base);
    const float4 kx4 = *reinterpret_cast<const float4*>(kx + base);
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
    const float4 dp4 = prev0 ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4*>(Dio + base);
    float dW, dE, kE3;
    quad_x_edges(Din, kx, d, kx4, base, i0, q, p, lane, dW, dE, kE3);
    quad_cells<STOREF>(d, kx4, dS, dN, dB, dF, kyS, kyN, kzB, kzF, r4, dp4, dW, dE, kE3, south, north, back, front,
                       i0, p, s, bc, Dio, F, base, act);
}

// The same update for the quad column t (q, j) on planes k0 .. k1-1 in turn:
// the plane below and the plane above (D and the z-faces) stay in registers
// from one plane to the next, so a plane loads nine quads instead of twelve
// and the quad's indices are computed once.  Bit-identical to mixed_quad
// plane by plane (same neighbours, same quad_cells).
template <bool STOREF>
__device__ __forceinline__ void mixed_quad_march(const float* __restrict__ Din, float* __restrict__ Dio,
                                                 const float* __restrict__ Rin, const float* __restrict__ kx,
                                                 const float* __restrict__ ky, const float* __restrict__ kz,
                                                 float* __restrict__ F, const MixScal& s, bool prev0,
                                                 const BC6<float>& bc, const Pad& p, int t, int k0, int k1, int lane,
                                                 bool live) {
    const int q = t % p.nq;
    int j = t / p.nq;
    const bool act = live && j < p.ny;
    if (j >= p.ny) j = p.ny - 1;
    const int i0 = 4 * q;
    const bool south = j > 0, north = j < p.ny - 1;
    long long base = i0 + (long long)p.PX * j + p.plane * k0;
    float4 d = *reinterpret_cast<const float4*>(Din + base);
    float4 dB = k0 > 0 ? *reinterpret_cast<const float4*>(Din + base - p.plane) : d;
    float4 kzB = *reinterpret_cast<const float4*>(kz + base);
    for (int k = k0; k < k1; ++k, base += p.plane) {
        const bool back = k > 0, front = k < p.nz - 1;
        const float4 dF = front ? *reinterpret_cast<const float4*>(Din + base + p.plane) : d;
        const float4 kzF = *reinterpret_cast<const float4*>(kz + base + p.plane);
        const float4 kx4 = *reinterpret_cast<const float4*>(kx + base);
        const float4 dS = south ? *reinterpret_cast<const float4*>(Din + base - p.PX) : d;
        const float4 dN = north ? *reinterpret_cast<const float4*>(Din + base + p.PX) : d;
        const float4 kyS = *reinterpret_cast<const float4*>(ky + base);
        const float4 kyN = *reinterpret_cast<const float4*>(ky + base + p.PX);
        const float4 r4 = *reinterpret_cast<const float4*>(Rin + base);
        const float4 dp4 = prev0 ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4*>(Dio + base);
        float dW, dE, kE3;
        quad_x_edges(Din, kx, d, kx4, base, i0, q, p, lane, dW, dE, kE3);
        quad_cells<STOREF>(d, kx4, dS, dN, dB, dF, kyS, kyN, kzB, kzF, r4, dp4, dW, dE, kE3, south, north, back,
                           front, i0, p, s, bc, Dio, F, base, act);
        dB = d;
        d = dF;
        kzB = kzF;
    }
}
// Launch shape of k_mixed_inner: 64-thread blocks, 16 per SM (64 registers,
// half the SM's threads).  Measured at 255^3: 76.4 us per iteration against
// 77.0 (128 x 8), 77.9 (32 x 32) and 78.1 (256 x 4); fewer registers spill,
// more (72, fewer blocks) are slower.
#ifndef HT3D_MIX_BS
#define HT3D_MIX_BS 64
#endif
#ifndef HT3D_MIX_MINB
#define HT3D_MIX_MINB 16
#endif
// One instance: thread t of plane k = blockIdx.y handles quad t of the plane.
template <bool STOREF>
__global__ void __launch_bounds__(HT3D_MIX_BS, HT3D_MIX_MINB) k_mixed_inner(const float* __restrict__ Din, float* __restrict__ Dio,
                                                        const float* __restrict__ Rin, const float* __restrict__ kx,
                                                        const float* __restrict__ ky, const float* __restrict__ kz,
                                                        float* __restrict__ F, MixScal s, int prev0, BC6<float> bc,
                                                        Pad p) {
    mixed_quad<STOREF>(Din, Dio, Rin, kx, ky, kz, F, s, prev0 != 0, bc, p, blockIdx.x * blockDim.x + threadIdx.x,
                       blockIdx.y, threadIdx.x & 31);
}

// ---------------------------------------------------------------------------
// Two inner iterations per pass (temporal blocking).  A CTA of TB_Y warps
// owns a column tile of TB_X x TB_Y cells (its "halo tile"): warp w is row
// y0 + w, lane l the quad of cells x0 + 4l .. x0 + 4l + 3, as in
// k_mixed_inner.  Marching through a chunk of zchunk planes it computes
//   A: iteration n on every cell of the tile and on one cell past each end
//      of its rows (the cells x0 - 1 and x0 + TB_X of every row, all of
//      them computed by warp 0, one per lane), plane p;
//   B: iteration n+1 on the cells of the inner rows (warps 1..TB_Y-2) of
//      plane p-1 from D' of planes p-2 (registers), p-1 (own quad in
//      registers, x-neighbours by warp shuffles or the end cells,
//      y-neighbours from shared memory) and p (registers).
// Halo cells (one cell in x, one row in y, one plane before and after the
// chunk) are computed by both neighbouring CTAs.  Every field is read once
// per pass and D', D'' are written once each (the next pass needs both: D''
// and its previous correction D'); both go to buffers the pass does not
// read, since the halo reads neighbouring cells' D and Dprev.  Iteration B's
// Dprev is iteration A's input D, already in registers, and B's face
// conductivities and residual are A's, carried in registers from the plane
// before.  Both iterations use mixed_cell, so the result is bit-identical to
// two k_mixed_inner launches.
//
// The inputs of plane p (D over the tile plus one ring, kx, ky, kz, Rin,
// Dprev) are brought into shared memory by TMA tensor copies (one thread
// issues six 3-D box loads per plane, completing on the plane's mbarrier) two
// planes ahead, in a ring of TB_STAGES planes.  Every box covers columns
// x0 - 4 .. x0 + TB_X + 3 (TMA wants 16-byte aligned x: x0 is a multiple of 4); elements
// outside the arrays are zero-filled.  Every thread reads its quads with
// 16-byte shared loads.  Every mbarrier wait is bounded: on timeout the CTA
// records HT3D_ERR_TIMEOUT in *err, waits (bounded) for its copies in flight
// and returns.
// ---------------------------------------------------------------------------
#ifndef HT3D_TB_Y
#define HT3D_TB_Y 16
#endif
constexpr int TB_LANES = 32, TB_X = 4 * TB_LANES, TB_Y = HT3D_TB_Y, TB_STAGES = 3;
constexpr int TB_OX = TB_X, TB_OY = TB_Y - 2;  // cells of a tile that iteration B updates
constexpr int TB_W = TB_X + 8;                 // every box: columns x0 - 4 .. x0 + TB_X + 3
constexpr unsigned kTbWaitLimit = 1u << 22;
constexpr int kTbRd = 3 * TB_Y * TB_X;  // floats of the three A-result planes (and of the three 1 / diag planes)

struct __align__(128) TbStage {
    float D[TB_Y + 2][TB_W];    // rows y0-1 .. y0+TB_Y
    float pad0[(128 - ((TB_Y + 2) * TB_W * 4) % 128) % 128 / 4];
    float kx[TB_Y][TB_W];       // rows y0 .. y0+TB_Y-1
    float pad1[(128 - (TB_Y * TB_W * 4) % 128) % 128 / 4];
    float ky[TB_Y + 1][TB_W];   // rows y0 .. y0+TB_Y
    float pad2[(128 - ((TB_Y + 1) * TB_W * 4) % 128) % 128 / 4];
    float kz[TB_Y][TB_W];
    float pad3[(128 - (TB_Y * TB_W * 4) % 128) % 128 / 4];
    float R[TB_Y][TB_W];
    float pad4[(128 - (TB_Y * TB_W * 4) % 128) % 128 / 4];
    float Dp[TB_Y][TB_W];       // previous correction
    float pad5[(128 - (TB_Y * TB_W * 4) % 128) % 128 / 4];
};
constexpr unsigned kTbStageBytes = 4u * TB_W * ((TB_Y + 2) + TB_Y + (TB_Y + 1) + 3 * TB_Y);
static_assert(offsetof(TbStage, kx) % 128 == 0 && offsetof(TbStage, ky) % 128 == 0 &&
                  offsetof(TbStage, kz) % 128 == 0 && offsetof(TbStage, R) % 128 == 0 &&
                  offsetof(TbStage, Dp) % 128 == 0 && sizeof(TbStage) % 128 == 0,
              "TMA destinations must be 128-byte aligned");
static_assert((TB_W * 4) % 16 == 0 && TB_W <= 256,
              "TMA box rows must be whole 16-byte units of at most 256 elements");

struct TbMaps {  // tensor maps of one pass (by value, in the constant bank)
    CUtensorMap D, kx, ky, kz, R, Dp;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, unsigned limit = kTbWaitLimit) {
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// Coefficients of a quad (face conductivities and residual) and its input
// correction: what iteration B at a plane reuses from iteration A there.
struct QuadIn {
    float4 kW, kS, kN, kB, kF, r, xc;
    float kE3;  // east face of the quad's last cell
};

// One iteration on a quad: the four cells of mixed_quad with the same ghost
// rules (i0, j, k: the quad's first cell; neighbours passed in).  HAVE_RD:
// the cells' 1 / diag are given in rd4; else they are computed and returned
// in rd4 (iteration A hands them to iteration B, whose cells and face
// conductivities are the same).
template <bool HAVE_RD>
__device__ __forceinline__ void pair_quad(const QuadIn& c, float4 xp, float dW, float dE, float4 xs4, float4 xn4,
                                          float4 xb4, float4 xf4, int i0, int j, int k, const Pad& p,
                                          const BC6<float>& bc, const MixScal& s, float _dx2, float _dy2, float _dz2,
                                          float4& rd4, float4& xout, float4& fout) {
    const bool south = j > 0, north = j < p.ny - 1, back = k > 0, front = k < p.nz - 1;
    float o[4], of[4], rd[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int i = i0 + m;
        const float xc = c4(c.xc, m);
        const float xw = (i == 0) ? hghost(bc, 0, xc) : (m == 0 ? dW : c4(c.xc, m - 1));
        const float xe = (i == p.nx - 1) ? hghost(bc, 1, xc) : (m == 3 ? dE : c4(c.xc, m + 1));
        const float xs = south ? c4(xs4, m) : hghost(bc, 2, xc);
        const float xn = north ? c4(xn4, m) : hghost(bc, 3, xc);
        const float xb = back ? c4(xb4, m) : hghost(bc, 4, xc);
        const float xf = front ? c4(xf4, m) : hghost(bc, 5, xc);
        const float kE = m == 3 ? c.kE3 : c4(c.kW, m + 1);
        rd[m] = HAVE_RD ? c4(rd4, m)
                        : mixed_rdiag(c4(c.kW, m), kE, c4(c.kS, m), c4(c.kN, m), c4(c.kB, m), c4(c.kF, m), s.cX,
                                      _dx2, _dy2, _dz2);
        mixed_cell_rd(xc, xw, xe, xs, xn, xb, xf, c4(c.kW, m), kE, c4(c.kS, m), c4(c.kN, m), c4(c.kB, m),
                      c4(c.kF, m), c4(c.r, m), c4(xp, m), rd[m], s.mom, s.dh2, s.cX, _dx2, _dy2, _dz2, of[m], o[m]);
    }
    if (i0 + 4 > p.nx) {  // the row's last quad: its padding cells stay zero
#pragma unroll
        for (int m = 0; m < 4; ++m)
            if (i0 + m >= p.nx) o[m] = of[m] = 0.f;
    }
    if (!HAVE_RD) rd4 = make_float4(rd[0], rd[1], rd[2], rd[3]);
    xout = make_float4(o[0], o[1], o[2], o[3]);
    fout = make_float4(of[0], of[1], of[2], of[3]);
}

// One iteration on one cell (the end cells of a tile's rows), with the ghost
// rules of mixed_quad; sh points at the cell in a stage's D tile.
__device__ __forceinline__ float pair_cell(const float* d, const float* kxr, const float* kyr, float kB, float kF,
                                           float r, float xp, float xb, float xf, int i, int j, int k, const Pad& p,
                                           const BC6<float>& bc, const MixScal& s, float _dx2, float _dy2,
                                           float _dz2) {
    const float xc = d[0];
    const float xw = (i == 0) ? hghost(bc, 0, xc) : d[-1];
    const float xe = (i == p.nx - 1) ? hghost(bc, 1, xc) : d[1];
    const float xs = (j > 0) ? d[-TB_W] : hghost(bc, 2, xc);
    const float xn = (j < p.ny - 1) ? d[TB_W] : hghost(bc, 3, xc);
    const float xbb = (k > 0) ? xb : hghost(bc, 4, xc);
    const float xff = (k < p.nz - 1) ? xf : hghost(bc, 5, xc);
    float f, x;
    mixed_cell(xc, xw, xe, xs, xn, xbb, xff, kxr[0], kxr[1], kyr[0], kyr[TB_W], kB, kF, r, xp, s.mom, s.dh2, s.cX,
               s._dx, s._dy, s._dz, _dx2, _dy2, _dz2, f, x);
    return x;
}

template <bool STOREF>
__global__ void __launch_bounds__(TB_LANES* TB_Y, TB_Y <= 8 ? 2 : 1) k_mixed_inner2(const __grid_constant__ TbMaps maps,
                                                                    const float* __restrict__ Din,
                                                                    float* __restrict__ D1out,
                                                                    float* __restrict__ D2out, float* __restrict__ F,
                                                                    MixScal s, BC6<float> bc, Pad p, int zchunk,
                                                                    int* __restrict__ err, int skip_plane,
                                                                    unsigned detect_limit) {
    extern __shared__ unsigned char tb_raw[];
    unsigned char* base = tb_raw + ((128 - (smem_u32(tb_raw) & 127)) & 127);
    TbStage* st = reinterpret_cast<TbStage*>(base);
    float* xbuf = reinterpret_cast<float*>(base + sizeof(TbStage) * TB_STAGES);  // A's result, three planes
    // A's 1 / diag, three planes, at kTbRd floats after the result of the same plane
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + sizeof(TbStage) * TB_STAGES + sizeof(float) * 2 * kTbRd);
    __shared__ int abort_flag;
    // A's end-cell results of the last three planes ([plane % 3][west, east][row]):
    // B of plane pl - 1 reads slot (pl - 1) % 3 after the CTA barrier of plane
    // pl, and warp 0 writes it again at plane pl + 2, after the barrier of
    // plane pl + 1, which every warp passes after its B of plane pl - 1
    __shared__ float ebuf[3][2][TB_Y];
    const int lane = threadIdx.x, ty = threadIdx.y, tid = lane + TB_LANES * ty;
    const int x0 = blockIdx.x * TB_OX, y0 = blockIdx.y * TB_OY - 1;  // tile origin (x0 % 4 == 0)
    const int i0 = x0 + 4 * lane, j = y0 + ty;
    const bool rowin = j >= 0 && j < p.PY && i0 < p.PX;  // quad inside the padded array
    const bool inner = i0 < p.nx && j >= 0 && j < p.ny && ty >= 1 && ty <= TB_Y - 2;
    // end cells (iteration A only): the columns x0 - 1 and x0 + TB_X of the
    // tile's rows, all computed by warp 0, which runs no iteration B: lane l
    // takes row l % TB_Y, its west end for l < TB_Y and its east end above.
    // Their results reach the warps' iteration B through ebuf.
    static_assert(2 * TB_Y <= TB_LANES, "one end cell per lane of warp 0");
    const bool endc = ty == 0 && lane < 2 * TB_Y;
    const int er = lane % TB_Y, ej = y0 + er;  // its row
    const int eside = lane < TB_Y ? 0 : 1;
    const int ie = eside ? x0 + TB_X : x0 - 1;
    const int ce = eside ? TB_X + 4 : 3;  // its column in the boxes
    const int k0 = blockIdx.z * zchunk, k1 = min(p.nz, k0 + zchunk);
    const int pa0 = max(k0 - 1, 0);
    const int plast = min(k1 + 1, p.nz);  // last staged plane (plane nz: its bottom z-faces)
    const float _dx2 = __fmul_rn(s._dx, s._dx), _dy2 = __fmul_rn(s._dy, s._dy), _dz2 = __fmul_rn(s._dz, s._dz);
    // this thread's offsets inside a stage (fixed over planes)
    const int oD = (ty + 1) * TB_W + 4 + 4 * lane;  // D, quad centre
    const int oK = ty * TB_W + 4 + 4 * lane;        // kx, ky (south), kz, R, Dp
    const int oC = ty * TB_X + 4 * lane;            // the A-result planes
    auto issue = [&](int k) {  // one thread: the six boxes of plane k into slot k % TB_STAGES
        if (k == skip_plane) return;  // HT3D_TUNE_WAIT_TEST only: never issued, its wait runs out
        TbStage& S = st[k % TB_STAGES];
        uint64_t* b = &bar[k % TB_STAGES];
        mbar_expect_tx(b, kTbStageBytes);
        tma_load3(&S.D[0][0], &maps.D, x0 - 4, y0 - 1, k, b);
        tma_load3(&S.kx[0][0], &maps.kx, x0 - 4, y0, k, b);
        tma_load3(&S.ky[0][0], &maps.ky, x0 - 4, y0, k, b);
        tma_load3(&S.kz[0][0], &maps.kz, x0 - 4, y0, k, b);
        tma_load3(&S.R[0][0], &maps.R, x0 - 4, y0, k, b);
        tma_load3(&S.Dp[0][0], &maps.Dp, x0 - 4, y0, k, b);
    };
    if (tid == 0) {
        abort_flag = 0;
        for (int q = 0; q < TB_STAGES; ++q) mbar_init(&bar[q], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        issue(pa0);
        if (pa0 + 1 <= plast) issue(pa0 + 1);
    }
    int issued = min(pa0 + 1, plast);  // last plane whose copies are in flight or done
    const TbStage* S0 = &st[pa0 % TB_STAGES];
    const TbStage* S1 = &st[(pa0 + 1) % TB_STAGES];
    const TbStage* S2 = &st[(pa0 + 2) % TB_STAGES];
    // A's result of plane pl goes to buffer pl % 3; B reads plane pl - 1's.  A of
    // plane pl + 2 reuses the buffer B of plane pl - 1 reads, and every warp has
    // finished that B before the CTA barrier that plane pl + 1's A precedes.
    float* xw_ = xbuf + (pa0 % 3) * TB_Y * TB_X + oC;
    float* xr_ = xbuf + ((pa0 + 2) % 3) * TB_Y * TB_X + oC;
    float* xn_ = xbuf + ((pa0 + 1) % 3) * TB_Y * TB_X + oC;
    const long long colo = i0 + (long long)p.PX * j;
    float* outD1 = D1out + colo + p.plane * (long long)(pa0 - 1);
    float* outD2 = D2out + colo + p.plane * (long long)(pa0 - 1);
    float* outF = F + colo + p.plane * (long long)(pa0 - 1);
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 dm1 = (pa0 > 0 && rowin) ? *reinterpret_cast<const float4*>(Din + p.plane * (pa0 - 1) + colo) : z4;
    // the end cell's D at the plane before, and its A result at the plane before
    const bool endin = endc && ej >= 0 && ej < p.PY && ie >= 0 && ie < p.PX;
    float em1 = (pa0 > 0 && endin) ? Din[p.plane * (pa0 - 1) + ie + (long long)p.PX * ej] : 0.f;
    float4 dpm = z4, dpc = z4;  // A's result at planes pl - 2 and pl - 1
    QuadIn cb{};                // A's inputs at plane pl - 1 (B's coefficients)
    for (int pl = pa0; pl <= k1; ++pl) {
        if (pl + 2 <= plast) {
            // slot (pl + 2) % 3 was last read by iteration A of planes pl - 1 and
            // pl - 2, which every warp finished before the CTA barrier of the
            // previous plane.  Lane 0 of the last warp issues (that warp runs
            // no iteration B; warp 0 computes the end cells).
            if (tid == TB_LANES * (TB_Y - 1)) {
                // order the earlier generic reads of this slot before the async-proxy writes
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(pl + 2);
            }
            issued = pl + 2;
        }
        // planes pl and pl + 1 have landed (phase = number of earlier uses of the
        // slot): every lane waits on the barriers itself, which also makes the
        // copied data visible to it.  Plane pl was waited for as plane pl + 1
        // of the previous iteration (pl <= plast throughout).  A warp runs at
        // most one plane ahead of another (one CTA barrier per plane), so the
        // phase it waits for is always the slot's next one.
        bool ok = true;
        if (pl == pa0) ok = mbar_wait_bounded(&bar[pl % TB_STAGES], 0, detect_limit);
        if (pl + 1 <= plast)
            ok = ok && mbar_wait_bounded(&bar[(pl + 1) % TB_STAGES], ((pl + 1 - pa0) / TB_STAGES) & 1, detect_limit);
        if (!ok) abort_flag = 1;
        // ---- A: iteration n at plane pl, every quad of the halo tile
        QuadIn ca{};
        float4 da = z4;
        if (ok && pl < p.nz) {
            const float* d0 = &S0->D[0][0] + oD;
            ca.xc = lds4(d0);
            ca.kW = lds4(&S0->kx[0][0] + oK);
            ca.kE3 = (&S0->kx[0][0])[oK + 4];
            ca.kS = lds4(&S0->ky[0][0] + oK);
            ca.kN = lds4(&S0->ky[0][0] + oK + TB_W);
            ca.kB = lds4(&S0->kz[0][0] + oK);
            ca.kF = lds4(&S1->kz[0][0] + oK);
            ca.r = lds4(&S0->R[0][0] + oK);
            const float4 xp = lds4(&S0->Dp[0][0] + oK);
            const float4 xs4 = lds4(d0 - TB_W), xn4 = lds4(d0 + TB_W);
            const float4 xf4 = lds4(&S1->D[0][0] + oD);
            float4 fa, rda;
            pair_quad<false>(ca, xp, d0[-1], d0[4], xs4, xn4, dm1, xf4, i0, j, pl, p, bc, s, _dx2, _dy2, _dz2, rda, da,
                             fa);
            dm1 = ca.xc;
            *reinterpret_cast<float4*>(xw_) = da;
            *reinterpret_cast<float4*>(xw_ + kTbRd) = rda;
        }
        if (ok && pl < p.nz && endc) {
            const int oe = er * TB_W + ce;
            const float* de = &S0->D[0][0] + (er + 1) * TB_W + ce;
            ebuf[pl % 3][eside][er] =
                pair_cell(de, &S0->kx[0][0] + oe, &S0->ky[0][0] + oe, (&S0->kz[0][0])[oe], (&S1->kz[0][0])[oe],
                          (&S0->R[0][0])[oe], (&S0->Dp[0][0])[oe], em1, (&S1->D[0][0])[(er + 1) * TB_W + ce], ie, ej,
                          pl, p, bc, s, _dx2, _dy2, _dz2);
            em1 = de[0];
        }
        __syncthreads();
        if (abort_flag) {  // a wait gave up: every thread leaves here
            if (tid == 0) {
                atomicExch(err, HT3D_ERR_TIMEOUT);
                // every copy issued must land before the CTA's shared memory is released
                for (int q = pl; q <= issued; ++q)
                    if (q != skip_plane) mbar_wait_bounded(&bar[q % TB_STAGES], ((q - pa0) / TB_STAGES) & 1);
            }
            __syncthreads();
            return;
        }
        // ---- B: iteration n+1 at plane pl - 1 on the inner quads
        // every lane takes part in the shuffles
        float bW = __shfl_up_sync(0xffffffffu, dpc.w, 1);
        float bE = __shfl_down_sync(0xffffffffu, dpc.x, 1);
        // slot (pl - 1) % 3, written by warp 0 at plane pl - 1 (only read when
        // B runs: the first plane of a chunk has no such slot yet)
        if (lane == 0 && pl - 1 >= k0) bW = ebuf[(pl + 2) % 3][0][ty];
        if (lane == TB_LANES - 1 && pl - 1 >= k0) bE = ebuf[(pl + 2) % 3][1][ty];
        if (pl - 1 >= k0 && inner) {
            const int q = pl - 1;
            QuadIn c = cb;
            const float4 xprev = c.xc;  // B's previous correction: A's input
            c.xc = dpc;
            float4 xb2, fb, rdb = lds4(xr_ + kTbRd);
            pair_quad<true>(c, xprev, bW, bE, lds4(xr_ - TB_X), lds4(xr_ + TB_X), dpm, da, i0, j, q, p, bc, s, _dx2,
                            _dy2, _dz2, rdb, xb2, fb);
            *reinterpret_cast<float4*>(outD1) = dpc;
            *reinterpret_cast<float4*>(outD2) = xb2;
            if (STOREF) *reinterpret_cast<float4*>(outF) = fb;
        }
        outD1 += p.plane;
        outD2 += p.plane;
        outF += p.plane;
        dpm = dpc;
        dpc = da;
        cb = ca;
        const TbStage* t = S0;
        S0 = S1;
        S1 = S2;
        S2 = t;
        float* u = xr_;
        xr_ = xw_;
        xw_ = xn_;
        xn_ = u;
    }
}
constexpr size_t kTbSmem = 128 + sizeof(TbStage) * TB_STAGES + sizeof(float) * 2 * kTbRd + 8 * TB_STAGES;

// cuTensorMapEncodeTiled, fetched from the driver at run time (no libcuda link)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)f;
        else
            cudaGetLastError();
    });
    return fn;
}
// map of a padded FP32 field: (PX, PY, nz+1) elements, boxes width x rows x 1
bool tb_map(CUtensorMap* m, const float* field, const Pad& P, unsigned width, unsigned rows) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)P.PX, (cuuint64_t)P.PY, (cuuint64_t)P.nz + 1};
    const cuuint64_t strides[2] = {(cuuint64_t)P.PX * 4, (cuuint64_t)P.plane * 4};
    const cuuint32_t box[3] = {width, rows, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)field, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Batched inner iteration over an ensemble of independent instances.  One
// launch covers up to kEnsMaxPerLaunch members: the concatenation of their
// grids: BS quads per block over each member's (quad, row, plane) range.
// The members' records travel by value in the kernel parameters (constant bank), so a
// block finds its member and fields without a dependent global load before
// its first field load.
// ---------------------------------------------------------------------------
struct EnsInner {
    float* D[2];  // correction ping-pong: read D[parity], Dprev / write D[parity ^ 1]
    const float* Rin;
    float* F;
    const float* kx;
    const float* ky;
    const float* kz;
    Pad P;
    MixScal s;
    BC6<float> bc;
};
constexpr int kEnsMaxPerLaunch = 120;
struct EnsLaunch {
    int n;                                // members in this launch
    int nblk;                             // blocks of this launch
    int block0[kEnsMaxPerLaunch + 1];     // first block of each member (block0[n] = nblk)
    int quads[kEnsMaxPerLaunch];          // quads per plane (nq * ny) of each member
    int nbq[kEnsMaxPerLaunch];            // z-march kernel: blocks per plane (ceil(quads / BS))
    EnsInner rec[kEnsMaxPerLaunch];
};
static_assert(sizeof(EnsLaunch) <= 32000, "batched launch parameters exceed the 32 KB kernel parameter space");

template <bool STOREF, int BS>
__global__ void __launch_bounds__(BS) k_ens_inner(const __grid_constant__ EnsLaunch L, int parity, int prev0) {
    // member of this block: binary search of the block offsets
    int lo = 0, hi = L.n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((int)blockIdx.x >= L.block0[mid]) lo = mid;
        else hi = mid;
    }
    const EnsInner& e = L.rec[lo];
    // the member's quads in (quad, row, plane) order, BS per block across planes
    // (fewer than 2^30 quads per member: 32-bit unsigned arithmetic)
    const unsigned tg = (unsigned)(blockIdx.x - L.block0[lo]) * BS + threadIdx.x;
    const unsigned pq = (unsigned)L.quads[lo];  // quads per plane
    int k = (int)(tg / pq);
    const int t = (int)(tg - (unsigned)k * pq);
    const bool live = k < e.P.nz;
    if (!live) k = e.P.nz - 1;
    mixed_quad<STOREF>(e.D[parity], e.D[parity ^ 1], e.Rin, e.kx, e.ky, e.kz, e.F, e.s, prev0 != 0, e.bc, e.P, t, k,
                       threadIdx.x & 31, live);
}

// The same iteration with each thread marching one quad column over KC planes
// (mixed_quad_march): a member's blocks are nbq per plane range (BS quads of
// a plane each) times ceil(nz / KC) plane ranges.
template <bool STOREF, int BS, int KC>
__global__ void __launch_bounds__(BS) k_ens_march(const __grid_constant__ EnsLaunch L, int parity, int prev0) {
    int lo = 0, hi = L.n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((int)blockIdx.x >= L.block0[mid]) lo = mid;
        else hi = mid;
    }
    const EnsInner& e = L.rec[lo];
    const int lb = (int)blockIdx.x - L.block0[lo];
    const int nbq = L.nbq[lo];
    const int bz = lb / nbq, bq = lb - bz * nbq;
    const int pq = L.quads[lo];
    const int t = bq * BS + (int)threadIdx.x;
    const bool live = t < pq;
    const int k0 = bz * KC, k1 = min(e.P.nz, k0 + KC);
    mixed_quad_march<STOREF>(e.D[parity], e.D[parity ^ 1], e.Rin, e.kx, e.ky, e.kz, e.F, e.s, prev0 != 0, e.bc, e.P,
                             live ? t : pq - 1, k0, k1, threadIdx.x & 31, live);
}

// FP64 check / refresh iteration of the mixed solver (see above).  FP64
// fields in the reference layout, FP32 fields in the padded layout.  The fold
// X + D and the residual are FP64; the quantities stored in FP32 (F, the
// momentum F0 = (Dprev - D) / dtau_prev, the next correction) are formed in
// FP32, and the Rayleigh-quotient terms are summed per thread in FP32 (they
// only estimate lambda_min).  Dio holds Dprev on entry (prev0: Dprev = 0) and
// receives the next correction -dtau F0', whose own previous correction is 0
// (D has been folded into X).  CHECK = false (a refresh between the
// reference's checks) skips the check sums and the FP64 F.
template <bool CHECK>
__global__ void __launch_bounds__(TX* TY, 3) k_mixed_check(
    const double* __restrict__ Xin, double* __restrict__ Xout, const float* __restrict__ Din, float* __restrict__ Dio,
    const double* __restrict__ R, const double* __restrict__ kx, const double* __restrict__ ky,
    const double* __restrict__ kz, const double* __restrict__ invPC, float* __restrict__ F32,
    double* __restrict__ F64, float* __restrict__ Rin, DyrelScal s, MixScal s32, int prev0, BC6<double> bc, Pad p,
    int zchunk, double* __restrict__ partials) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int i = x0 + tx;
    const int j = y0 + ty;
    const int k0 = blockIdx.z * zchunk;
    const int k1 = min(nz, k0 + zchunk);
    double acc[3] = {0.0, 0.0, 0.0};
    float rq_num = 0.f, rq_den = 0.f;
    // The folds X + D of a plane's tile and of its ring (the row before and
    // after the tile, the column before and after it) go to shared memory,
    // two planes deep: a cell's x- and y-neighbours are read there instead
    // of being folded again (one fold per cell instead of five; the ring
    // takes three warp instructions).  Every thread of the block runs the
    // plane loop for the barriers; cells outside the grid do no work.
    __shared__ double xt[2][TY + 2][TX + 2];
    const bool act = i < nx && j < ny;
    const int n1 = nx + 2, n2 = ny + 2;
    const long long pl = (long long)n1 * n2, cpl = (long long)nx * ny, pp = p.plane;
    // fold of inner cell (ii, jj) at plane kk
    auto fold_at = [&](int ii, int jj, int kk) {
        return Xin[(ii + 1) + (long long)n1 * (jj + 1) + pl * (kk + 1)] +
               (double)Din[ii + (long long)p.PX * jj + pp * kk];
    };
    // ring cell of this thread, if any: warp 0 the row y0 - 1, warp TY - 1 the
    // row y0 + TY, warp 1 the columns x0 - 1 (lanes 0 .. TY-1) and x0 + TX
    // (lanes TY .. 2 TY - 1)
    int ri = -1, rj = -1, rs = 0, rc = 0;  // cell, and its slot in the tile
    if (ty == 0 && i < nx && y0 > 0) { ri = i; rj = y0 - 1; rs = 0; rc = tx + 1; }
    else if (ty == TY - 1 && i < nx && y0 + TY < ny) { ri = i; rj = y0 + TY; rs = TY + 1; rc = tx + 1; }
    else if (ty == 1 && tx < TY && x0 > 0 && y0 + tx < ny) { ri = x0 - 1; rj = y0 + tx; rs = tx + 1; rc = 0; }
    else if (ty == 1 && tx >= TY && tx < 2 * TY && x0 + TX < nx && y0 + tx - TY < ny) {
        ri = x0 + TX; rj = y0 + tx - TY; rs = tx - TY + 1; rc = TX + 1;
    }
    if (k0 < k1) {
        const int ic = act ? i : 0, jc = act ? j : 0;  // cells outside the grid address cell (0, 0)
        const long long col = (ic + 1) + (long long)n1 * (jc + 1);
        const long long pcol = ic + (long long)p.PX * jc;
        const double* xcol = Xin + col;
        const float* dcol = Din + pcol;
        double* ocol = Xout + col;
        const long long ccol = ic + (long long)nx * jc;
        const double* kxcol = kx + ic + (long long)(nx + 1) * jc;
        const double* kycol = ky + ic + (long long)nx * jc;
        const double* kzcol = kz + ccol;
        auto fold = [&](long long e, long long pe) { return xcol[e] + (double)dcol[pe]; };
        double xc = act ? fold(pl * (k0 + 1), pp * k0) : 0.0;
        double xb = (!act || k0 == 0) ? ghost(bc, 4, xc) : fold(pl * k0, pp * (k0 - 1));
        double qB = act ? -kzcol[cpl * k0] * (s._dz * (xc - xb)) : 0.0;
        for (int k = k0; k < k1; ++k) {
            const int b = k & 1;
            // the plane's per-cell loads go out before the barrier, so their
            // latency overlaps it (each address is read, and later written,
            // by this thread alone)
            const long long e = pl * (k + 1), pe = pp * k;
            const long long c = ccol + cpl * k, pc = pcol + pe;
            const long long fxo = (long long)(nx + 1) * ny * k, fyo = (long long)nx * (ny + 1) * k;
            double gR = 0.0, gI = 0.0, gkF = 0.0, gkW = 0.0, gkE = 0.0, gkS = 0.0, gkN = 0.0, xnext = 0.0;
            float gDp = 0.f, gD = 0.f, gF = 0.f;
            if (act) {
                gR = R[c];
                gI = invPC[c];
                gkF = kzcol[cpl * (k + 1)];
                gkW = kxcol[fxo];
                gkE = kxcol[fxo + 1];
                gkS = kycol[fyo];
                gkN = kycol[fyo + nx];
                gDp = prev0 ? 0.f : Dio[pc];
                gD = dcol[pe];
                if (CHECK) gF = F32[pc];
                if (k != nz - 1) xnext = fold(e + pl, pe + pp);
            }
            xt[b][ty + 1][tx + 1] = xc;
            if (ri >= 0) xt[b][rs][rc] = fold_at(ri, rj, k);
            __syncthreads();  // also orders the reads of plane k - 2 (same buffer) before these writes
            if (act) {
                const double xf = (k == nz - 1) ? ghost(bc, 5, xc) : xnext;
                const double xw = (i == 0) ? ghost(bc, 0, xc) : xt[b][ty + 1][tx];
                const double xe = (i == nx - 1) ? ghost(bc, 1, xc) : xt[b][ty + 1][tx + 2];
                const double xs = (j == 0) ? ghost(bc, 2, xc) : xt[b][ty][tx + 1];
                const double xn = (j == ny - 1) ? ghost(bc, 3, xc) : xt[b][ty + 2][tx + 1];
                const double qF = -gkF * (s._dz * (xf - xc));
                const double qW = -gkW * (s._dx * (xc - xw));
                const double qE = -gkE * (s._dx * (xe - xc));
                const double qS = -gkS * (s._dy * (xc - xs));
                const double qN = -gkN * (s._dy * (xn - xc));
                const double fu = gR + s.cX * xc + s._dx * (qE - qW) + s._dy * (qN - qS) + s._dz * (qF - qB);
                const double f = fu * gI;
                const float f32 = (float)f;
                const float f0old = __fdiv_rn(__fsub_rn(gDp, gD), s32.dtau_prev);
                const float f0 = __fmaf_rn(s32.h1, f0old, __fmul_rn(s32.h2, f32));
                const float d = __fmul_rn(s32.dtau, f0);
                if (CHECK) {
                    acc[0] += fabs(fu);
                    rq_num = __fmaf_rn(-d, __fsub_rn(f32, gF), rq_num);
                    rq_den = __fmaf_rn(d, d, rq_den);
                    F64[c] = f;
                }
                F32[pc] = f32;
                Rin[pc] = (float)fu;
                Dio[pc] = -d;
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
    }
    if (!CHECK) return;
    acc[1] = (double)rq_num;
    acc[2] = (double)rq_den;
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

// The momentum after the last update, F0 = (Dprev - D) / dtau_prev (Dprev
// null: the correction was just folded, Dprev = 0), into a reference cell array.
__global__ void k_unpack_f0(double* __restrict__ dst, const float* __restrict__ D, const float* __restrict__ Dprev,
                            float dtau_prev, Pad p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= p.nx || j >= p.ny || k >= p.nz) return;
    const long long pe = i + (long long)p.PX * j + p.plane * k;
    const float dp = Dprev ? Dprev[pe] : 0.f;
    dst[i + (long long)p.nx * (j + (long long)p.ny * k)] = (double)__fdiv_rn(__fsub_rn(dp, D[pe]), dtau_prev);
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
    void count(int iterations = 1) { if (on) launches += iterations; }
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
    NvtxRange range("ht3d DYREL solve (mixed)");
    const long long n = (long long)nx * ny * nz;
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    const Pad P = make_pad(nx, ny, nz);
    HT3D_REQUIRE(P.size < (1LL << 31), "grid too large for the padded FP32 layout");
    const size_t pbytes = sizeof(float) * (size_t)P.size;
    double* invPC = (double*)ht3d_scratch(ctx, SLOT_PC, sizeof(double) * n);
    double* X2 = (double*)ht3d_scratch(ctx, SLOT_X2, sizeof(double) * nex);
    // correction buffers: the current D and its previous correction, plus two
    // more for the two-iteration passes (which write neither buffer they read)
    // two iterations per pass: always for an explicit z-chunk (>= 2); by default
    // (1) where the pass pays: grids of 2^21 cells or more whose x extent fills
    // its 128-cell tiles to 3/4 or more (smaller grids run faster one iteration
    // per launch: the pass's tiles would be mostly empty and its set-up is per solve)
    const int tiles_x = (nx + 127) / 128;
    const bool want_pairs = ctx->mixed_temporal >= 2 ||
                            (ctx->mixed_temporal == 1 && n >= (1LL << 21) && 4LL * nx >= 3LL * 128 * tiles_x);
    float* Dbuf[4] = {(float*)ht3d_scratch(ctx, SLOT_F32_X, pbytes), (float*)ht3d_scratch(ctx, SLOT_F32_X2, pbytes),
                      want_pairs ? (float*)ht3d_scratch(ctx, SLOT_F32_D3, pbytes) : nullptr,
                      want_pairs ? (float*)ht3d_scratch(ctx, SLOT_F32_D4, pbytes) : nullptr};
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
    HT3D_LAUNCH(ctx, k_dyrel_setup_fast, gc, b2, 0, kx, ky, kz, cX, 1.0 / (dx * dx), 1.0 / (dy * dy), 1.0 / (dz * dz),
                nx, ny, nz, invPC, parts);
    HT3D_LAUNCH(ctx, (k_reduce_partials<RED_MAX, 1>), 1, 1024, 0, parts, (int)(gc.x * gc.y * gc.z), dres);
    for (float* a : {Dbuf[0], Dbuf[1], Dbuf[2], Dbuf[3], Fs, Rin, kx32, ky32, kz32})
        if (a) HT3D_CUDA(cudaMemsetAsync(a, 0, pbytes, ctx->stream));
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
    const dim3 ib(HT3D_MIX_BS), ig((unsigned)(((long long)P.nq * ny + HT3D_MIX_BS - 1) / HT3D_MIX_BS), (unsigned)nz);
    // two iterations per pass (k_mixed_inner2) inside runs of inner iterations
    bool pairs = want_pairs;
    int zc = ctx->mixed_temporal >= 2 ? ctx->mixed_temporal : 0;
    const int tiles = ((nx + TB_OX - 1) / TB_OX) * ((ny + TB_OY - 1) / TB_OY);
    if (!zc) {  // fewest waves x (chunk + the two planes iteration A adds)
        const long long slots = (long long)ctx->num_sms * (TB_Y <= 8 ? 2 : 1);  // resident CTAs
        long long best = -1;
        for (int c = 8; c <= 64; ++c) {
            const long long ctas = (long long)tiles * ((nz + c - 1) / c);
            const long long cost = (ctas + slots - 1) / slots * (std::min(c, nz) + 2);
            if (best < 0 || cost < best) best = cost, zc = c;
        }
    }
    const dim3 tb(TB_LANES, TB_Y), tg((nx + TB_OX - 1) / TB_OX, (ny + TB_OY - 1) / TB_OY, (nz + zc - 1) / zc);
    TbMaps mk;                       // conductivity and residual maps
    CUtensorMap mapD[4], mapP[4];    // each correction buffer as a pass's D (with its ring) and as its Dprev
    int* derr = nullptr;
    if (pairs) {
        pairs = tb_map(&mk.kx, kx32, P, TB_W, TB_Y) && tb_map(&mk.ky, ky32, P, TB_W, TB_Y + 1) &&
                tb_map(&mk.kz, kz32, P, TB_W, TB_Y) && tb_map(&mk.R, Rin, P, TB_W, TB_Y);
        for (int q = 0; q < 4 && pairs; ++q)
            pairs = tb_map(&mapD[q], Dbuf[q], P, TB_W, TB_Y + 2) && tb_map(&mapP[q], Dbuf[q], P, TB_W, TB_Y);
    }
    if (pairs) {
        static_assert(kTbSmem <= 227 * 1024, "staging ring exceeds the shared memory of a CTA");
        HT3D_CUDA(cudaFuncSetAttribute(k_mixed_inner2<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTbSmem));
        HT3D_CUDA(cudaFuncSetAttribute(k_mixed_inner2<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTbSmem));
        derr = (int*)ht3d_scratch(ctx, SLOT_AUX0, sizeof(int) * 16);
        HT3D_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), ctx->stream));
    }
    InnerTimer timer(ctx);
    double* xcur = X;
    double* xnxt = X2;
    int cur = 0, prv = 1;            // Dbuf indices of D and of its previous correction
    bool prev0 = true;               // the previous correction is 0 (start, or D just folded into X)
    double dtau_prev = S.dtau;       // dtau of the update that produced D
    DyrelCheck C;
    int it_done = 0;
    bool last_fp64 = false;  // the last iteration ran the FP64 kernel (check or refresh)
    bool last_chk = false;   // ... and was a check (which writes the FP64 F)
    const int nmax = n_iter_fixed > 0 ? n_iter_fixed : prm->nitmax;
    const int refresh_every = ctx->mixed_refresh;
    auto is_fp64 = [&](int it) {
        return is_check(it, prm->nitout) || (refresh_every > 0 && it % refresh_every == 0);
    };
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
        const MixScal s32 = mix_scal(sc, dtau_prev);
        if (chk || refresh) {
            timer.end();
            if (chk)
                HT3D_LAUNCH(ctx, k_mixed_check<true>, LC.grid, LC.block, 0, xcur, xnxt, Dbuf[cur], Dbuf[prv], R, kx, ky,
                            kz, invPC, Fs, F, Rin, sc, s32, prev0 ? 1 : 0, bc, P, LC.zchunk, parts);
            else
                HT3D_LAUNCH(ctx, k_mixed_check<false>, LC.grid, LC.block, 0, xcur, xnxt, Dbuf[cur], Dbuf[prv], R, kx,
                            ky, kz, invPC, Fs, F, Rin, sc, s32, prev0 ? 1 : 0, bc, P, LC.zchunk, parts);
            std::swap(xcur, xnxt);
            std::swap(cur, prv);  // the new correction sits in the former Dprev buffer
            prev0 = true;
        } else {
            timer.begin();
            // this run of inner iterations ends at run_end; a run that ends the
            // solve keeps its last iteration single (the final fold needs the
            // correction before the last iteration)
            int run_end = iter;
            while (run_end < nmax && !is_fp64(run_end + 1)) ++run_end;
            const int pair_end = run_end == nmax ? run_end - 1 : run_end;
            const int left = pair_end - iter + 1;
            // a pass starts only on a steady iteration (Dprev stored, mom = h1)
            if (pairs && !prev0 && dtau_prev == sc.dtau && left >= 2 && left % 2 == 0) {
                const bool storef2 = iter + 1 == nmax || is_check(iter + 2, prm->nitout);
                int o1 = -1, o2 = -1;  // the two buffers the pass does not read
                for (int q = 0; q < 4; ++q)
                    if (q != cur && q != prv) (o1 < 0 ? o1 : o2) = q;
                TbMaps mp = mk;
                mp.D = mapD[cur];
                mp.Dp = mapP[prv];
                // HT3D_TUNE_WAIT_TEST: this pass skips one plane's copies and detects with a short limit
                const int skip = ctx->wait_test > 0 ? ctx->wait_test - 1 : -1;
                const unsigned lim = ctx->wait_test > 0 ? (1u << 12) : kTbWaitLimit;
                ctx->wait_test = 0;
                if (storef2)
                    HT3D_LAUNCH(ctx, k_mixed_inner2<true>, tg, tb, kTbSmem, mp, Dbuf[cur], Dbuf[o1], Dbuf[o2], Fs, s32,
                                bch, P, zc, derr, skip, lim);
                else
                    HT3D_LAUNCH(ctx, k_mixed_inner2<false>, tg, tb, kTbSmem, mp, Dbuf[cur], Dbuf[o1], Dbuf[o2], Fs,
                                s32, bch, P, zc, derr, skip, lim);
                prv = o1;
                cur = o2;
                timer.count(2);
                ++iter;  // the pass did iterations iter and iter + 1
            } else {
                if (storef)
                    HT3D_LAUNCH(ctx, k_mixed_inner<true>, ig, ib, 0, Dbuf[cur], Dbuf[prv], Rin, kx32, ky32, kz32, Fs,
                                s32, prev0 ? 1 : 0, bch, P);
                else
                    HT3D_LAUNCH(ctx, k_mixed_inner<false>, ig, ib, 0, Dbuf[cur], Dbuf[prv], Rin, kx32, ky32, kz32, Fs,
                                s32, prev0 ? 1 : 0, bch, P);
                std::swap(cur, prv);
                timer.count();
            }
            prev0 = false;
        }
        dtau_prev = sc.dtau;
        it_done = iter;
        last_fp64 = chk || refresh;
        last_chk = chk;
        if (chk) {
            HT3D_LAUNCH(ctx, (k_reduce_partials<RED_SUM, 3>), 1, 1024, 0, parts, (int)LC.nblocks, dres);
            ht3d_fetch_results(ctx, dres, 3);
            if (C.update(S, prm, ctx->h_result[0], ctx->h_result[1], ctx->h_result[2], (double)n, iter,
                         n_iter_fixed <= 0))
                break;
        }
    }
    timer.end();
    // final fold of the correction into the FP64 solution
    HT3D_LAUNCH(ctx, k_mixed_fold, gc, b2, 0, xcur, Dbuf[cur], last_fp64 ? nullptr : Dbuf[prv], bc, P);
    if (xcur != X) {
        dim3 g((nx + 2 + 31) / 32, (ny + 2 + 7) / 8, nz + 2);
        HT3D_LAUNCH(ctx, k_copy_ex_faces<double>, g, b2, 0, X, xcur, nx, ny, nz);
    }
    HT3D_LAUNCH(ctx, k_unpack_f0, gc, b2, 0, F0, Dbuf[cur], prev0 ? nullptr : Dbuf[prv], (float)dtau_prev, P);
    if (!last_chk) HT3D_LAUNCH(ctx, k_unpack, gc, b2, 0, F, Fs, P);
    if (derr) {  // a bounded wait of k_mixed_inner2 gave up
        int herr = 0;
        HT3D_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
        if (herr) C.status = herr;  // the root cause: later NaN checks follow from the aborted pass
    }
    timer.collect();
    C.fill(st, S, it_done);
    return C.status;
}


// ---------------------------------------------------------------------------
// Batched mixed solve (see ensemble_internal.cuh).  The schedule, the
// kernels and the reductions of every instance are those of
// ht3d_dyrel_solve_mixed; only the FP32 inner iterations of all instances
// share one launch per group of kEnsMaxPerLaunch members (or one CUDA graph
// of kEnsGraphIters iterations).
// ---------------------------------------------------------------------------
namespace {

struct Carve {
    char* base;
    size_t off = 0;
    template <typename T>
    T* take(size_t count) {
        off = (off + 255) & ~(size_t)255;
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += sizeof(T) * (count ? count : 1);
        return p;
    }
};

// Tile shapes of the batched iteration the autotuner chooses from: threads
// per block and planes per thread (0: one plane, k_ens_inner; KC: a z-march
// over KC planes, k_ens_march).
struct EnsCfg {
    int bs, kc;
};
constexpr int kEnsNCfg = 6;
constexpr int kEnsNCfgMax = 8;  // tile shapes the CUDA-graph key holds (3 bits)
static_assert(kEnsNCfg <= kEnsNCfgMax, "tile shapes must fit the graph key");
constexpr EnsCfg kEnsCfg[kEnsNCfg] = {{64, 0}, {128, 0}, {256, 0}, {64, 8}, {128, 8}, {128, 16}};
constexpr int kEnsGraphIters = 16;
constexpr int kEnsTuneRounds = 2;  // timed launches per tile shape

template <bool STOREF>
void ens_launch_raw(cudaStream_t st, int cfg, const EnsLaunch& L, int parity, int prev0) {
    const unsigned g = (unsigned)L.nblk;
    switch (cfg) {
    case 0: k_ens_inner<STOREF, 64><<<g, 64, 0, st>>>(L, parity, prev0); break;
    case 1: k_ens_inner<STOREF, 128><<<g, 128, 0, st>>>(L, parity, prev0); break;
    case 2: k_ens_inner<STOREF, 256><<<g, 256, 0, st>>>(L, parity, prev0); break;
    case 3: k_ens_march<STOREF, 64, 8><<<g, 64, 0, st>>>(L, parity, prev0); break;
    case 4: k_ens_march<STOREF, 128, 8><<<g, 128, 0, st>>>(L, parity, prev0); break;
    default: k_ens_march<STOREF, 128, 16><<<g, 128, 0, st>>>(L, parity, prev0); break;
    }
}

template <bool STOREF>
int ens_launch_all(cudaStream_t st, int cfg, const std::vector<EnsLaunch>& groups, int parity, int prev0) {
    for (const EnsLaunch& L : groups) ens_launch_raw<STOREF>(st, cfg, L, parity, prev0);
    return (int)groups.size();
}

struct EnsHost {
    Pad P;
    IterLaunch LC;
    double* invPC;
    double* X2;
    float* f32[7];  // Da, Db, F, Rin, kx, ky, kz
    double* xcur;
    double* xnxt;
    DyrelState S;
    DyrelScal sc;
    double dtau_prev;  // dtau of the update that produced the current correction
    BC6<double> bc;
    BC6<float> bch;
    bool used, active, last_fp64, last_chk;
    int it_done;
    DyrelCheck C;
};

unsigned long long mix_sig(unsigned long long h, unsigned long long v) {
    return (h ^ v) * 0x100000001b3ULL + 0x9e3779b97f4a7c15ULL;
}

// Key of the captured graphs: the launch groups' version (unique per build of
// the groups on this context) and the tile shape, exactly (a hash of the two
// could let a later solve replay an earlier solve's graph, whose member
// records and scratch layout are stale).
unsigned long long graph_sig(unsigned long long version, int cfg) {
    return (version << 3) | (unsigned long long)cfg;
}

// Captures the two graphs (windows starting on parity 0 and 1) of the
// current launch groups; false when the stream cannot be captured.
bool ens_capture(ht3d_ctx* ctx, unsigned long long sig, int cfg, const std::vector<EnsLaunch>& groups) {
    if (ctx->ens_graph_sig == sig && ctx->ens_graph[0] && ctx->ens_graph[1]) return true;
    for (auto& g : ctx->ens_graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    ctx->ens_graph_sig = 0;
    for (int p = 0; p < 2; ++p) {
        if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        for (int g = 0; g < kEnsGraphIters; ++g) ens_launch_all<false>(ctx->stream, cfg, groups, (p + g) & 1, 0);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
        if (e != cudaSuccess || !graph) {
            cudaGetLastError();
            return false;
        }
        const cudaError_t ei = cudaGraphInstantiate(&ctx->ens_graph[p], graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            cudaGetLastError();
            ctx->ens_graph[p] = nullptr;
            return false;
        }
    }
    ctx->ens_graph_sig = sig;
    return true;
}

}  // namespace

void ht3d_ensemble_solve_mixed(ht3d_ctx* ctx, EnsSolveInst* in, int n) {
    NvtxRange range("ht3d batched DYREL solve");
    std::vector<EnsHost> H(n);
    int nitout = 0, nitmax = 0, nused = 0;
    for (int q = 0; q < n; ++q) {
        H[q].used = in[q].status == 0;
        if (!H[q].used) continue;
        HT3D_REQUIRE(in[q].prm && in[q].prm->nitout > 0 && in[q].prm->nitmax > 0, "DYREL parameters");
        if (nused == 0) {
            nitout = in[q].prm->nitout;
            nitmax = in[q].prm->nitmax;
        }
        HT3D_REQUIRE(in[q].prm->nitout == nitout && in[q].prm->nitmax == nitmax,
                     "ensemble instances must share nitout and nitmax");
        ++nused;
    }
    if (nused == 0) return;

    // ---- per-instance scratch (FP64 check fields, padded FP32 fields)
    auto carve_solve = [&](Carve& c) {
        for (int q = 0; q < n; ++q) {
            if (!H[q].used) continue;
            EnsHost& h = H[q];
            const EnsSolveInst& I = in[q];
            h.P = make_pad(I.nx, I.ny, I.nz);
            h.invPC = c.take<double>((size_t)I.nx * I.ny * I.nz);
            h.X2 = c.take<double>((size_t)(I.nx + 2) * (I.ny + 2) * (I.nz + 2));
            for (auto& f : h.f32) f = c.take<float>((size_t)h.P.size);
        }
    };
    long long maxparts = 1;
    for (int q = 0; q < n; ++q) {
        if (!H[q].used) continue;
        const EnsSolveInst& I = in[q];
        ht3d_check_dims(I.nx, I.ny, I.nz, 1);
        HT3D_REQUIRE(I.X && I.R && I.kx && I.ky && I.kz && I.F && I.F0 && I.bc_type6 && I.bc_val6, "null argument");
        const Pad P = make_pad(I.nx, I.ny, I.nz);
        HT3D_REQUIRE(P.size < (1LL << 31), "grid too large for the padded FP32 layout");
        HT3D_REQUIRE(((long long)P.nq * I.ny * I.nz + kEnsCfg[0].bs - 1) / kEnsCfg[0].bs < (1LL << 30),
                     "member too large for the batched launch");
        H[q].LC = iter_launch(ctx, I.nx, I.ny, I.nz, HT3D_DYREL_ZMARCH);
        maxparts = std::max(maxparts, std::max<long long>(H[q].LC.nblocks, (long long)((I.nx + 31) / 32) *
                                                                               ((I.ny + 7) / 8) * I.nz));
    }
    {
        Carve dry{nullptr};
        carve_solve(dry);
        Carve real{(char*)ht3d_scratch(ctx, SLOT_ENS_SOLVE, dry.off)};
        carve_solve(real);
    }
    double* dres = (double*)ht3d_scratch(ctx, SLOT_ENS_TAB, sizeof(double) * 4 * (size_t)n);
    double* parts = (double*)ht3d_scratch(ctx, SLOT_PARTIALS, sizeof(double) * 3 * maxparts);
    // pinned staging of the results
    const size_t hbytes = sizeof(double) * 4 * (size_t)n;
    HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_ens_bytes < hbytes) {
        if (ctx->h_ens) HT3D_CUDA(cudaFreeHost(ctx->h_ens));
        ctx->h_ens = nullptr;
        ctx->h_ens_bytes = 0;
        HT3D_CUDA(cudaMallocHost(&ctx->h_ens, hbytes));
        ctx->h_ens_bytes = hbytes;
    }
    double* hres = (double*)ctx->h_ens;

    // ---- set-up of every instance (Gershgorin bound, FP32 copies)
    const dim3 b2(32, 8, 1);
    for (int q = 0; q < n; ++q) {
        EnsHost& h = H[q];
        if (!h.used) continue;
        const EnsSolveInst& I = in[q];
        const int nx = I.nx, ny = I.ny, nz = I.nz;
        for (int f = 0; f < 6; ++f) {
            HT3D_REQUIRE(I.bc_type6[f] == HT3D_BC_NEUMANN || I.bc_type6[f] == HT3D_BC_DIRICHLET,
                         "face BC type must be 0 or 1");
            h.bc.dir[f] = h.bch.dir[f] = I.bc_type6[f];
            h.bc.val2[f] = 2.0 * I.bc_val6[f];
            h.bch.val2[f] = 0.0f;
        }
        const dim3 gc((nx + 31) / 32, (ny + 7) / 8, nz);
        HT3D_LAUNCH(ctx, k_dyrel_setup_fast, gc, b2, 0, I.kx, I.ky, I.kz, I.cX, 1.0 / (I.dx * I.dx),
                    1.0 / (I.dy * I.dy), 1.0 / (I.dz * I.dz), nx, ny, nz, h.invPC, parts);
        HT3D_LAUNCH(ctx, (k_reduce_partials<RED_MAX, 1>), 1, 1024, 0, parts, (int)(gc.x * gc.y * gc.z), dres + q);
        const size_t pbytes = sizeof(float) * (size_t)h.P.size;
        for (float* a : h.f32) HT3D_CUDA(cudaMemsetAsync(a, 0, pbytes, ctx->stream));
        HT3D_LAUNCH(ctx, k_pack, dim3((nx + 1 + 31) / 32, (ny + 7) / 8, nz), b2, 0, h.f32[4], I.kx, nx + 1, ny, nz, h.P);
        HT3D_LAUNCH(ctx, k_pack, dim3((nx + 31) / 32, (ny + 1 + 7) / 8, nz), b2, 0, h.f32[5], I.ky, nx, ny + 1, nz, h.P);
        HT3D_LAUNCH(ctx, k_pack, dim3((nx + 31) / 32, (ny + 7) / 8, nz + 1), b2, 0, h.f32[6], I.kz, nx, ny, nz + 1, h.P);
    }
    HT3D_CUDA(cudaMemcpyAsync(hres, dres, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int q = 0; q < n; ++q) {
        EnsHost& h = H[q];
        if (!h.used) continue;
        const EnsSolveInst& I = in[q];
        dyrel_init_params(I.prm, hres[q], h.S);
        h.sc.cX = I.cX;
        h.sc._dx = 1.0 / I.dx;
        h.sc._dy = 1.0 / I.dy;
        h.sc._dz = 1.0 / I.dz;
        h.sc.h1 = h.S.h1;
        h.sc.h2 = h.S.h2;
        h.sc.dtau = h.S.dtau;
        h.dtau_prev = h.S.dtau;
        h.xcur = I.X;
        h.xnxt = h.X2;
        h.active = true;
        h.last_fp64 = false;
        h.last_chk = false;
        h.it_done = 0;
        h.C = DyrelCheck();
    }

    // ---- launch groups of the members still iterating, for each block size;
    // rebuilt when a check changes the members' scalars or stops a member
    std::vector<EnsLaunch> groups[kEnsNCfg];
    unsigned long long version = 0;
    // members in launch order: largest first, so the blocks of the members
    // with the most work start first and the launch's tail is made of small
    // members' blocks (longest-processing-time-first); results do not depend
    // on the order
    std::vector<int> order;
    for (int q = 0; q < n; ++q)
        if (H[q].used) order.push_back(q);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long long)in[a].nx * in[a].ny * in[a].nz > (long long)in[b].nx * in[b].ny * in[b].nz;
    });
    auto build_groups = [&]() {
        version = ++ctx->ens_version;
        for (int c = 0; c < kEnsNCfg; ++c) {
            groups[c].clear();
            const int bs = kEnsCfg[c].bs, kc = kEnsCfg[c].kc;
            for (int q : order) {
                const EnsHost& h = H[q];
                if (!h.active) continue;
                if (groups[c].empty() || groups[c].back().n == kEnsMaxPerLaunch) {
                    groups[c].emplace_back();
                    std::memset(&groups[c].back(), 0, sizeof(EnsLaunch));
                }
                EnsLaunch& L = groups[c].back();
                const long long pq = (long long)h.P.nq * in[q].ny;
                const long long nbq = (pq + bs - 1) / bs;
                const long long nb_q = kc == 0 ? (pq * in[q].nz + bs - 1) / bs : nbq * ((in[q].nz + kc - 1) / kc);
                if ((long long)L.nblk + nb_q >= (1LL << 31) - 1) {  // start a new group before the count overflows
                    groups[c].emplace_back();
                    std::memset(&groups[c].back(), 0, sizeof(EnsLaunch));
                }
                EnsLaunch& G = groups[c].back();
                const int m = G.n++;
                G.block0[m] = G.nblk;
                G.quads[m] = (int)pq;
                G.nbq[m] = (int)nbq;
                G.nblk += (int)nb_q;
                G.block0[m + 1] = G.nblk;
                EnsInner& e = G.rec[m];
                e.D[0] = h.f32[0];
                e.D[1] = h.f32[1];
                e.F = h.f32[2];
                e.Rin = h.f32[3];
                e.kx = h.f32[4];
                e.ky = h.f32[5];
                e.kz = h.f32[6];
                e.P = h.P;
                e.s = mix_scal(h.sc, h.dtau_prev);
                e.bc = h.bch;
            }
        }
    };
    build_groups();

    // ---- block size: fixed, tuned earlier for this ensemble shape, or tuned now
    unsigned long long shape = 0xcbf29ce484222325ULL;
    for (int q = 0; q < n; ++q)
        if (H[q].used) shape = mix_sig(mix_sig(mix_sig(mix_sig(shape, q), in[q].nx), in[q].ny), in[q].nz);
    int cfg = -1;
    auto cfg_of = [](int bs) { return bs == 64 ? 0 : (bs == 128 ? 1 : 2); };
    if (ctx->ens_tile) cfg = ctx->ens_tile - 1;
    else if (ctx->ens_block) cfg = cfg_of(ctx->ens_block);
    else if (ctx->ens_tune_key == shape && ctx->ens_tune_cfg) cfg = ctx->ens_tune_cfg - 1;
    bool tuning = cfg < 0;
    int tune_n = 0;
    if (tuning)
        while ((int)ctx->tune_events.size() < 2 * kEnsNCfg * kEnsTuneRounds) {
            cudaEvent_t ev;
            HT3D_CUDA(cudaEventCreate(&ev));
            ctx->tune_events.push_back(ev);
        }
    bool graphs = ctx->ens_graphs != 0;

    const int refresh_every = ctx->mixed_refresh;
    auto is_fp64 = [&](int it) { return is_check(it, nitout) || (refresh_every > 0 && it % refresh_every == 0); };
    auto is_storef = [&](int it) { return !is_fp64(it) && (it == nitmax || is_check(it + 1, nitout)); };
    InnerTimer timer(ctx);
    int nactive = nused;
    int prev0 = 1;  // the previous corrections are 0 (start, or D just folded): same for every member
    for (int iter = 1; iter <= nitmax && nactive > 0; ++iter) {
        const int parity = (iter - 1) & 1;  // correction buffer of every instance still iterating
        const bool chk = is_check(iter, nitout);
        if (is_fp64(iter)) {
            timer.end();
            for (int q = 0; q < n; ++q) {
                EnsHost& h = H[q];
                if (!h.active) continue;
                h.sc.h1 = h.S.h1;
                h.sc.h2 = h.S.h2;
                h.sc.dtau = h.S.dtau;
                const EnsSolveInst& I = in[q];
                const MixScal s32 = mix_scal(h.sc, h.dtau_prev);
                if (chk)
                    HT3D_LAUNCH(ctx, k_mixed_check<true>, h.LC.grid, h.LC.block, 0, h.xcur, h.xnxt, h.f32[parity],
                                h.f32[parity ^ 1], I.R, I.kx, I.ky, I.kz, h.invPC, h.f32[2], I.F, h.f32[3], h.sc, s32,
                                prev0, h.bc, h.P, h.LC.zchunk, parts);
                else
                    HT3D_LAUNCH(ctx, k_mixed_check<false>, h.LC.grid, h.LC.block, 0, h.xcur, h.xnxt, h.f32[parity],
                                h.f32[parity ^ 1], I.R, I.kx, I.ky, I.kz, h.invPC, h.f32[2], I.F, h.f32[3], h.sc, s32,
                                prev0, h.bc, h.P, h.LC.zchunk, parts);
                h.dtau_prev = h.sc.dtau;
                std::swap(h.xcur, h.xnxt);
                h.it_done = iter;
                h.last_fp64 = true;
                h.last_chk = chk;
                if (chk)
                    HT3D_LAUNCH(ctx, (k_reduce_partials<RED_SUM, 3>), 1, 1024, 0, parts, (int)h.LC.nblocks,
                                dres + 3 * q);
            }
            prev0 = 1;
        } else {
            timer.begin();
            const bool storef = is_storef(iter);
            int window = 1;
            if (!storef && !tuning && graphs && !prev0) {
                window = 0;
                while (window < kEnsGraphIters && iter + window <= nitmax && !is_fp64(iter + window) &&
                       !is_storef(iter + window))
                    ++window;
                if (window == kEnsGraphIters) {
                    graphs = ens_capture(ctx, graph_sig(version, cfg), cfg, groups[cfg]);
                    if (!graphs) window = 1;
                } else {
                    window = 1;
                }
            }
            if (window == kEnsGraphIters) {
                HT3D_CUDA(cudaGraphLaunch(ctx->ens_graph[parity], ctx->stream));
                ctx->launches += (unsigned long long)kEnsGraphIters * groups[cfg].size();
                for (int g = 0; g < kEnsGraphIters; ++g) timer.count();
            } else {
                int c = tuning ? 1 : cfg;
                const bool timed = tuning && !storef;
                if (timed) {
                    c = tune_n % kEnsNCfg;
                    HT3D_CUDA(cudaEventRecord(ctx->tune_events[2 * tune_n], ctx->stream));
                }
                const int nl = storef ? ens_launch_all<true>(ctx->stream, c, groups[c], parity, prev0)
                                      : ens_launch_all<false>(ctx->stream, c, groups[c], parity, prev0);
                ctx->launches += nl;
                timer.count();
                if (timed) {
                    HT3D_CUDA(cudaEventRecord(ctx->tune_events[2 * tune_n + 1], ctx->stream));
                    if (++tune_n == kEnsNCfg * kEnsTuneRounds) {
                        HT3D_CUDA(cudaEventSynchronize(ctx->tune_events[2 * tune_n - 1]));
                        float best = 0.f;
                        for (int cc = 0; cc < kEnsNCfg; ++cc) {
                            float sum = 0.f;
                            for (int r = 0; r < kEnsTuneRounds; ++r) {
                                float ms = 0.f;
                                const int t = r * kEnsNCfg + cc;
                                HT3D_CUDA(cudaEventElapsedTime(&ms, ctx->tune_events[2 * t], ctx->tune_events[2 * t + 1]));
                                sum += ms;
                            }
                            if (cc == 0 || sum < best) {
                                best = sum;
                                cfg = cc;
                            }
                        }
                        tuning = false;
                        ctx->ens_tune_key = shape;
                        ctx->ens_tune_cfg = cfg + 1;
                    }
                }
            }
            // the records hold mom = h1 dtau / dtau_prev: rebuild them when
            // that was the first iteration after a parameter update
            bool stale = false;
            for (int q = 0; q < n; ++q)
                if (H[q].active) {
                    H[q].it_done = iter + window - 1;
                    H[q].last_fp64 = false;
                    H[q].last_chk = false;
                    stale = stale || H[q].dtau_prev != H[q].sc.dtau;
                    H[q].dtau_prev = H[q].sc.dtau;
                }
            prev0 = 0;
            if (stale) build_groups();
            iter += window - 1;
        }
        if (chk) {
            HT3D_CUDA(cudaMemcpyAsync(hres, dres, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
            HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
            for (int q = 0; q < n; ++q) {
                EnsHost& h = H[q];
                if (!h.active) continue;
                const double nc = (double)in[q].nx * in[q].ny * in[q].nz;
                const bool stop =
                    h.C.update(h.S, in[q].prm, hres[3 * q], hres[3 * q + 1], hres[3 * q + 2], nc, iter, true);
                if (stop) {
                    h.active = false;
                    --nactive;
                }
                h.sc.h1 = h.S.h1;
                h.sc.h2 = h.S.h2;
                h.sc.dtau = h.S.dtau;
            }
            if (nactive > 0) build_groups();
        }
    }
    timer.end();
    // ---- final fold and outputs of every instance
    for (int q = 0; q < n; ++q) {
        EnsHost& h = H[q];
        if (!h.used) continue;
        const EnsSolveInst& I = in[q];
        const int nx = I.nx, ny = I.ny, nz = I.nz;
        const dim3 gc((nx + 31) / 32, (ny + 7) / 8, nz);
        const int dc = h.it_done & 1;  // current correction buffer after it_done iterations
        HT3D_LAUNCH(ctx, k_mixed_fold, gc, b2, 0, h.xcur, h.f32[dc], h.last_fp64 ? nullptr : h.f32[dc ^ 1], h.bc, h.P);
        if (h.xcur != I.X) {
            dim3 g((nx + 2 + 31) / 32, (ny + 2 + 7) / 8, nz + 2);
            HT3D_LAUNCH(ctx, k_copy_ex_faces<double>, g, b2, 0, I.X, h.xcur, nx, ny, nz);
        }
        HT3D_LAUNCH(ctx, k_unpack_f0, gc, b2, 0, I.F0, h.f32[dc], h.last_fp64 ? nullptr : h.f32[dc ^ 1],
                    (float)h.dtau_prev, h.P);
        if (!h.last_chk) HT3D_LAUNCH(ctx, k_unpack, gc, b2, 0, I.F, h.f32[2], h.P);
        h.C.fill(I.st, h.S, h.it_done);
        in[q].status = h.C.status;
    }
    timer.collect();
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
