// Internal definitions shared by the libht3d translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <stdexcept>

#include <nvtx3/nvToolsExt.h>  // header-only NVTX v3: named ranges for timeline profilers

#include "../../include/ht3d.h"

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
// A slot grows by free + malloc, so a pointer taken from a slot is invalid
// once anything asks the same slot for more bytes: each user below owns its
// slot for the duration of a call.
enum ScratchSlot {
    SLOT_PARTIALS = 0,  // solver check terms / per-block partials (double)
    SLOT_REDUCE,        // partials of ht3d_reduce_device (used between solver phases)
    SLOT_RESULT,        // final reduction results (double[64])
    SLOT_X2,            // ping-pong ghosted field
    SLOT_PC,            // Jacobi diagonal / inverse diagonal
    SLOT_G,             // Gershgorin ratios
    SLOT_SNAP,          // pre-launch snapshot for in-place boundary kernels
    SLOT_F32_X, SLOT_F32_X2, SLOT_F32_D3, SLOT_F32_R, SLOT_F32_PC, SLOT_F32_KX, SLOT_F32_KY, SLOT_F32_KZ,
    SLOT_F32_F, SLOT_F32_D4,
    SLOT_STEP_R, SLOT_STEP_F, SLOT_STEP_F0, SLOT_STEP_TY, SLOT_STEP_KX, SLOT_STEP_KY, SLOT_STEP_KZ,
    SLOT_WENO_T0, SLOT_WENO_T1, SLOT_WENO_T2, SLOT_WENO_V,
    SLOT_AUX0, SLOT_AUX1, SLOT_AUX2, SLOT_AUX3,
    SLOT_ENS_SOLVE,     // batched solve: per-instance FP64 and padded FP32 fields
    SLOT_ENS_TAB,       // batched solve: per-instance check results
    SLOT_ENS_STEP,      // ensemble step: per-instance residual, flux and conductivity fields
    SLOT_COUNT
};

struct ht3d_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sync_each_call = 1;
    int dyrel_variant = 0;                // thread layout of the fused DYREL iteration (0 = per precision)
    int mixed_refresh = 512;              // FP64 defect-correction cadence of the mixed solver
    int mixed_temporal = 1;               // mixed form: two inner iterations per pass (>= 2: z-chunk)
    int wait_test = 0;                    // > 0: the next pass skips plane wait_test - 1 (bounded-wait test)
    int time_inner = 0;                   // time the mixed solver's inner-iteration runs
    std::vector<cudaEvent_t> events;      // event pool of the inner-iteration timer
    double inner_ms = 0.0;                // accumulated device time of the timed runs
    unsigned long long inner_launches = 0;  // inner iterations inside them
    // batched ensemble solve
    int ens_block = 0;                    // threads per block of the batched kernel (0 = autotune)
    int ens_graphs = 1;                   // replay windows of inner iterations as CUDA graphs
    unsigned long long ens_tune_key = 0;  // ensemble signature the tuned block size belongs to
    int ens_tune_cfg = 0;                 // tuned tile shape of that ensemble (index + 1)
    int ens_tile = 0;                     // fixed tile shape of the batched iteration (index + 1, 0 = autotune)
    std::vector<cudaEvent_t> tune_events;
    unsigned long long ens_version = 0;   // bumped whenever the batched launch parameters change
    unsigned long long ens_graph_sig = 0; // launch parameters the captured graphs carry
    cudaGraphExec_t ens_graph[2] = {nullptr, nullptr};  // windows starting on parity 0 / 1
    void* h_ens = nullptr;                // pinned staging (instance records, results)
    size_t h_ens_bytes = 0;
    int num_sms = 152;
    unsigned long long launches = 0;
    std::string last_error;
    void* slot_ptr[SLOT_COUNT] = {};
    size_t slot_bytes[SLOT_COUNT] = {};
    double* h_result = nullptr;  // pinned, 64 doubles
};

// Named host range around a solver phase ("ht3d step_hrl", "ht3d thermal
// solve", ...), visible in timeline profilers; free when none is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct ht3d_error : public std::runtime_error {
    int code;
    ht3d_error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define HT3D_CUDA(call)                                                                          \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            throw ht3d_error(HT3D_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

#define HT3D_REQUIRE(cond, msg) \
    do {                        \
        if (!(cond)) throw ht3d_error(HT3D_ERR_ARG, msg); \
    } while (0)

// Runs `body` and converts exceptions into status codes; honours
// sync_each_call (reference @parallel calls are synchronous).
template <typename Fn>
static inline int ht3d_guard(ht3d_ctx* ctx, Fn&& body, bool sync = true) {
    if (!ctx) return HT3D_ERR_ARG;
    try {
        HT3D_CUDA(cudaSetDevice(ctx->device));
        int st = body();
        HT3D_CUDA(cudaGetLastError());
        if (sync && ctx->sync_each_call) HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
        return st;
    } catch (const ht3d_error& e) {
        ctx->last_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        ctx->last_error = e.what();
        return HT3D_ERR_CUDA;
    }
}

void* ht3d_scratch(ht3d_ctx* ctx, int slot, size_t bytes);

// every pointer argument is set (entry points reject NULL before any launch)
template <typename... P>
static inline bool all_nonnull(P... p) {
    return ((p != nullptr) && ...);
}

// ---------------------------------------------------------------------------
// Launch helpers
// ---------------------------------------------------------------------------
#define HT3D_LAUNCH(ctx, kern, grid, block, smem, ...)                         \
    do {                                                                       \
        kern<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);         \
        (ctx)->launches++;                                                     \
    } while (0)

// Phase codes (-1 immersed, 0 crust, 1 air, 2 fault, 3 pluton) are small
// integers stored as doubles.  Equality with a nonzero code is tested on the
// bit pattern: the same truth value as the FP64 comparison for every input,
// NaN included (a nonzero finite value has one representation), as an integer
// compare instead of an instruction on the FP64 pipe.
__device__ __forceinline__ bool ph_eq(double p, double code) {
    return __double_as_longlong(p) == __double_as_longlong(code);
}
__device__ __forceinline__ bool ph_abs_eq(double p, double code) {  // fabs(p) == code, code > 0
    return (__double_as_longlong(p) & 0x7fffffffffffffffLL) == __double_as_longlong(code);
}
// The sign the FP64 comparisons x < 0.0 and x > 0.0 see: -1, +1, or 0 for
// +-0 and NaN (both comparisons false), from the bit pattern with integer
// operations instead of two compares on the FP64 pipe.
__device__ __forceinline__ int cmp_sign(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long m = b & 0x7fffffffffffffffULL;
    if (m == 0ULL || m > 0x7ff0000000000000ULL) return 0;
    return (b >> 63) ? -1 : 1;
}

static inline dim3 grid3(long long n1, long long n2, long long n3, dim3 b) {
    return dim3((unsigned)((n1 + b.x - 1) / b.x), (unsigned)((n2 + b.y - 1) / b.y), (unsigned)((n3 + b.z - 1) / b.z));
}
static const dim3 kBlock3(32, 8, 1);

// Launch shape of the light per-cell kernels (a few loads and stores per
// cell): each kBlock3 block covers kZPer consecutive k planes of its 32 x 8
// tile, one (i, j) column per thread.  A 255^3 launch is then 8 k blocks
// instead of 65 k; scheduling 65 k one-cell blocks alone took about 60 us.
constexpr int kZPer = 8;
static inline dim3 grid3z(long long n1, long long n2, long long n3) {
    return dim3((unsigned)((n1 + 31) / 32), (unsigned)((n2 + 7) / 8), (unsigned)((n3 + kZPer - 1) / kZPer));
}
// Calls f(i, j, k) for this thread's cells of an n1 x n2 x n3 box (grid3z
// launch with kBlock3 blocks); a `return` in f skips one cell.
template <class F>
__device__ __forceinline__ void for_cells_z(int n1, int n2, int n3, F&& f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    const int k0 = blockIdx.z * kZPer;
#pragma unroll
    for (int kk = 0; kk < kZPer; ++kk)
        if (k0 + kk < n3) f(i, j, k0 + kk);
}

// Largest element count any array of an n^3 problem may have (n+6)^3 must fit
// 32-bit index arithmetic.
static inline void ht3d_check_dims(long long nx, long long ny, long long nz, int min_n = 1) {
    HT3D_REQUIRE(nx >= min_n && ny >= min_n && nz >= min_n, "grid dimensions below the minimum for this kernel");
    HT3D_REQUIRE((nx + 6) * (ny + 6) * (nz + 6) < (1LL << 31), "grid too large for 32-bit indexing");
}

// column-major (x fastest) index
__host__ __device__ static inline int ix3(int i, int j, int k, int n1, int n2) { return i + n1 * (j + n2 * k); }

// ---------------------------------------------------------------------------
// Reductions (deterministic: fixed block partition + fixed-order final pass)
// ---------------------------------------------------------------------------
enum RedOp { RED_SUM = 0, RED_SUM_ABS = 1, RED_MAX = 2, RED_MIN = 3, RED_MAX_ABS = 4 };

template <int OP>
__device__ __forceinline__ double red_identity() {
    return OP == RED_MAX ? -INFINITY : (OP == RED_MIN ? INFINITY : 0.0);
}
template <int OP>
__device__ __forceinline__ double red_combine(double a, double b) {
    if (OP == RED_MAX || OP == RED_MAX_ABS) return fmax(a, b);
    if (OP == RED_MIN) return fmin(a, b);
    return a + b;
}
template <int OP>
__device__ __forceinline__ double red_map(double x) {
    return (OP == RED_SUM_ABS || OP == RED_MAX_ABS) ? fabs(x) : x;
}

// Block-wide reduction of NV values per thread; result valid in thread 0.
// Uses warp shuffles then one shared-memory pass; blockDim.x*y*z <= 1024.
template <int OP, int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV]) {
    __shared__ double sh[32][NV];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nth = blockDim.x * blockDim.y * blockDim.z;
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] = red_combine<OP>(v[q], __shfl_down_sync(0xffffffffu, v[q], o));
    const int lane = tid & 31, warp = tid >> 5, nwarp = (nth + 31) >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[warp][q] = v[q];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double x = lane < nwarp ? sh[lane][q] : red_identity<OP>();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x = red_combine<OP>(x, __shfl_down_sync(0xffffffffu, x, o));
            v[q] = x;
        }
    }
}

// Final pass over `nparts` partials of NV interleaved values -> out[NV].
template <int OP, int NV>
__global__ void k_reduce_partials(const double* __restrict__ parts, int nparts, double* __restrict__ out) {
    double v[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = red_identity<OP>();
    for (int p = threadIdx.x; p < nparts; p += blockDim.x)
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q] = red_combine<OP>(v[q], parts[(size_t)p * NV + q]);
    block_reduce<OP, NV>(v);
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) out[q] = v[q];
}

// Reduce a strided/plain array on the device; writes result to
// device slot (double) at d_out and returns the host copy when sync.
double ht3d_reduce_device(ht3d_ctx* ctx, const double* a, long long n, int op, double* d_out);
// Same for float input (accumulated in double).
double ht3d_reduce_device_f32(ht3d_ctx* ctx, const float* a, long long n, int op, double* d_out);

// Read `count` doubles from device to the pinned host buffer (synchronises).
void ht3d_fetch_results(ht3d_ctx* ctx, const double* d_src, int count);
