// Allocation-free DYREL iteration.
//
// ht3d_dyrel_iterate needs one scratch field (the ping-pong target of the
// Jacobi-style update) and takes it from a context, which allocates device
// memory.  Some callers cannot allocate device memory at all: a host
// application that owns the whole device heap through its own pool or arena,
// or code running where memory management is frozen (for example between
// phases of a solver that must not perturb a measured memory footprint).
// ht3d_dyrel_iterate_noalloc gives them the same iteration without any
// allocation: the scratch field is a fixed, file-scope device array in this
// library, created once with the module on every device that loads it and
// kept until the process exits.
//
// Compiled with -fmad=false like the plain FP64 solver: the result is
// identical to ht3d_dyrel_iterate's.
#include <mutex>
#include <utility>

#include "dyrel_common.cuh"

namespace {

// Largest ghosted field, in doubles, the static scratch holds:
// (nx+2)(ny+2)(nz+2) <= 2^20 (8 MiB; e.g. 99^3 cells).
constexpr long long kNoallocMaxEx = 1LL << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_noalloc_scratch[kNoallocMaxEx];

// Device address of g_noalloc_scratch per device.  The symbol's name in host
// code is only a host-side stand-in, so the address is queried once per
// device with that device current.  cudaDeviceReset unloads the module, and
// the array may come back elsewhere: the cached address is then stale, so a
// process that resets a device must not call this entry point on it again.
double* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_setup_mutex;

int scratch_for_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HT3D_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return HT3D_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return HT3D_ERR_CUDA;
        }
        g_scratch_ptr[dev] = (double*)p;
    }
    *out = g_scratch_ptr[dev];
    return HT3D_OK;
}

// Launches through cudaLaunchKernel, whose return value is this launch's own
// status: an error left on the thread by someone else's earlier launch is
// neither reported as this call's nor cleared.
template <typename... P>
cudaError_t launch_exact(void (*kern)(P...), dim3 g, dim3 b, cudaStream_t st, P... args) {
    void* ptrs[] = {(void*)&args...};
    return cudaLaunchKernel((const void*)kern, g, b, ptrs, 0, st);
}
template <typename... P, typename... A>
cudaError_t launch(void (*kern)(P...), dim3 g, dim3 b, cudaStream_t st, A... args) {
    static_assert(sizeof...(P) == sizeof...(A), "argument count");
    return launch_exact<P...>(kern, g, b, st, static_cast<P>(args)...);
}

}  // namespace

extern "C" int ht3d_dyrel_iterate_noalloc(double* X_ex, const double* R, const double* kx, const double* ky,
                                          const double* kz, const double* PC, double* F0, double cX, double dx,
                                          double dy, double dz, const int* bc_type6, const double* bc_val6, double h1,
                                          double h2, double dtau, int n_iter, int nx, int ny, int nz, void* stream) {
    if (!X_ex || !R || !kx || !ky || !kz || !PC || !F0 || !bc_type6 || !bc_val6) return HT3D_ERR_ARG;
    if (nx < 1 || ny < 1 || nz < 1 || n_iter < 0) return HT3D_ERR_ARG;
    const long long nex = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    if (nex > kNoallocMaxEx) return HT3D_ERR_SCRATCH;
    BC6<double> bc;
    for (int f = 0; f < 6; ++f) {
        if (bc_type6[f] != HT3D_BC_NEUMANN && bc_type6[f] != HT3D_BC_DIRICHLET) return HT3D_ERR_ARG;
        bc.dir[f] = bc_type6[f];
        bc.val2[f] = 2.0 * bc_val6[f];
    }
    if (n_iter == 0) return HT3D_OK;  // nothing to do, nothing touched
    double* scratch = nullptr;
    const int s = scratch_for_current_device(&scratch);
    if (s != HT3D_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    const DyrelScalT<double> sc(DyrelScal{h1, h2, dtau, cX, 1.0 / dx, 1.0 / dy, 1.0 / dz});
    const dim3 blk(CX_, CY_, CZ_), grd((nx + CX_ - 1) / CX_, (ny + CY_ - 1) / CY_, (nz + CZ_ - 1) / CZ_);
    double* cur = X_ex;
    double* nxt = scratch;
    for (int it = 0; it < n_iter; ++it) {
        const cudaError_t e = launch(k_dyrel_cell<double, MODE_PLAIN>, grd, blk, st, cur, nxt, R, kx, ky, kz, PC, F0,
                                     (double*)nullptr, sc, bc, nx, ny, nz, (double*)nullptr);
        if (e != cudaSuccess) return HT3D_ERR_CUDA;
        std::swap(cur, nxt);
    }
    if (cur != X_ex) {
        const dim3 b(32, 8, 1), g((nx + 2 + 31) / 32, (ny + 2 + 7) / 8, nz + 2);
        if (launch(k_copy_ex_faces<double>, g, b, st, X_ex, cur, nx, ny, nz) != cudaSuccess) return HT3D_ERR_CUDA;
    }
    return HT3D_OK;
}
