// Context, scratch memory and deterministic reductions.
#include "ht3d_internal.cuh"

void* ht3d_scratch(ht3d_ctx* ctx, int slot, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (ctx->slot_bytes[slot] >= bytes) return ctx->slot_ptr[slot];
    if (ctx->slot_ptr[slot]) {
        // grow-only; the stream may still use the old buffer
        HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
        HT3D_CUDA(cudaFree(ctx->slot_ptr[slot]));
        ctx->slot_ptr[slot] = nullptr;
        ctx->slot_bytes[slot] = 0;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw ht3d_error(HT3D_ERR_NOMEM, std::string("cudaMalloc scratch failed: ") + cudaGetErrorString(e));
    }
    ctx->slot_ptr[slot] = p;
    ctx->slot_bytes[slot] = bytes;
    return p;
}

void ht3d_fetch_results(ht3d_ctx* ctx, const double* d_src, int count) {
    HT3D_CUDA(cudaMemcpyAsync(ctx->h_result, d_src, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->stream));
    HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
}

// grid-stride first pass: each block writes one partial
template <int OP, typename T>
__global__ void k_reduce_pass1(const T* __restrict__ a, long long n, double* __restrict__ parts) {
    double v[1] = {red_identity<OP>()};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride)
        v[0] = red_combine<OP>(v[0], red_map<OP>((double)a[t]));
    block_reduce<OP, 1>(v);
    if (threadIdx.x == 0) parts[blockIdx.x] = v[0];
}

template <typename T>
static double reduce_impl(ht3d_ctx* ctx, const T* a, long long n, int op, double* d_out) {
    const int threads = 256;
    long long want = (n + threads - 1) / threads;
    int blocks = (int)std::min<long long>(want, (long long)ctx->num_sms * 4);
    if (blocks < 1) blocks = 1;
    double* parts = (double*)ht3d_scratch(ctx, SLOT_REDUCE, sizeof(double) * 4096 * 4);
    double* out = d_out ? d_out : (double*)ht3d_scratch(ctx, SLOT_RESULT, sizeof(double) * 64);
    switch (op) {
#define RCASE(OPV)                                                                      \
    case OPV:                                                                           \
        HT3D_LAUNCH(ctx, (k_reduce_pass1<OPV, T>), blocks, threads, 0, a, n, parts);   \
        HT3D_LAUNCH(ctx, (k_reduce_partials<OPV, 1>), 1, 1024, 0, parts, blocks, out); \
        break;
        RCASE(RED_SUM) RCASE(RED_SUM_ABS) RCASE(RED_MAX) RCASE(RED_MIN) RCASE(RED_MAX_ABS)
#undef RCASE
        default: throw ht3d_error(HT3D_ERR_ARG, "unknown reduction op");
    }
    if (d_out) return 0.0;
    ht3d_fetch_results(ctx, out, 1);
    return ctx->h_result[0];
}

double ht3d_reduce_device(ht3d_ctx* ctx, const double* a, long long n, int op, double* d_out) {
    return reduce_impl<double>(ctx, a, n, op, d_out);
}
double ht3d_reduce_device_f32(ht3d_ctx* ctx, const float* a, long long n, int op, double* d_out) {
    return reduce_impl<float>(ctx, a, n, op, d_out);
}

extern "C" {

int ht3d_abi_version(void) { return HT3D_ABI_VERSION; }

const char* ht3d_status_string(int s) {
    switch (s) {
        case HT3D_OK: return "ok";
        case HT3D_ERR_ARG: return "invalid argument";
        case HT3D_ERR_CUDA: return "CUDA error";
        case HT3D_ERR_NAN: return "residual is NaN";
        case HT3D_ERR_DIVERGED: return "residual diverged (nF_rel > 100)";
        case HT3D_ERR_MAXITER: return "maximum iterations reached";
        case HT3D_ERR_TIMEOUT: return "bounded device wait timed out";
        case HT3D_ERR_NOMEM: return "out of device memory";
        case HT3D_ERR_SCRATCH: return "grid exceeds the 2^20-double static scratch of ht3d_dyrel_iterate_noalloc";
        case HT3D_ERR_IO: return "file could not be opened, written or read";
    }
    return "unknown status";
}

int ht3d_ctx_create(ht3d_ctx** out, int device, void* stream) {
    if (!out) return HT3D_ERR_ARG;
    *out = nullptr;
    ht3d_ctx* ctx = new (std::nothrow) ht3d_ctx();
    if (!ctx) return HT3D_ERR_NOMEM;
    ctx->device = device;
    try {
        HT3D_CUDA(cudaSetDevice(device));
        HT3D_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
        if (stream) {
            ctx->stream = (cudaStream_t)stream;
            ctx->own_stream = false;
        } else {
            HT3D_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
            ctx->own_stream = true;
        }
        HT3D_CUDA(cudaMallocHost((void**)&ctx->h_result, sizeof(double) * 64));
    } catch (const ht3d_error& e) {
        int c = e.code;
        if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return c;
    }
    *out = ctx;
    return HT3D_OK;
}

int ht3d_ctx_destroy(ht3d_ctx* ctx) {
    if (!ctx) return HT3D_ERR_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (int s = 0; s < SLOT_COUNT; ++s)
        if (ctx->slot_ptr[s]) cudaFree(ctx->slot_ptr[s]);
    if (ctx->h_result) cudaFreeHost(ctx->h_result);
    for (cudaEvent_t ev : ctx->events) cudaEventDestroy(ev);
    for (cudaEvent_t ev : ctx->tune_events) cudaEventDestroy(ev);
    for (cudaGraphExec_t g : ctx->ens_graph)
        if (g) cudaGraphExecDestroy(g);
    if (ctx->h_ens) cudaFreeHost(ctx->h_ens);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return HT3D_OK;
}

int ht3d_ctx_set_stream(ht3d_ctx* ctx, void* stream) {
    if (!ctx) return HT3D_ERR_ARG;
    return ht3d_guard(ctx, [&]() {
        HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
        if (ctx->own_stream) HT3D_CUDA(cudaStreamDestroy(ctx->stream));
        if (stream) {
            ctx->stream = (cudaStream_t)stream;
            ctx->own_stream = false;
        } else {
            HT3D_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
            ctx->own_stream = true;
        }
        return HT3D_OK;
    }, false);
}

int ht3d_ctx_set_sync(ht3d_ctx* ctx, int sync_each_call) {
    if (!ctx) return HT3D_ERR_ARG;
    ctx->sync_each_call = sync_each_call ? 1 : 0;
    return HT3D_OK;
}

int ht3d_ctx_set_tuning(ht3d_ctx* ctx, int key, int value) {
    if (!ctx) return HT3D_ERR_ARG;
    if (key == HT3D_TUNE_DYREL_VARIANT) {
        if (value != 0 && value != HT3D_DYREL_ZMARCH && value != HT3D_DYREL_CELL) return HT3D_ERR_ARG;
        ctx->dyrel_variant = value;
        return HT3D_OK;
    }
    if (key == HT3D_TUNE_MIXED_REFRESH) {
        if (value < 0) return HT3D_ERR_ARG;
        ctx->mixed_refresh = value;
        return HT3D_OK;
    }
    if (key == HT3D_TUNE_ENS_BLOCK) {
        if (value != 0 && value != 64 && value != 128 && value != 256) return HT3D_ERR_ARG;
        ctx->ens_block = value;
        return HT3D_OK;
    }
    if (key == HT3D_TUNE_ENS_TILE) {
        if (value < 0 || value > 6) return HT3D_ERR_ARG;
        ctx->ens_tile = value;
        return HT3D_OK;
    }
    if (key == HT3D_TUNE_ENS_GRAPH) {
        if (value != 0 && value != 1) return HT3D_ERR_ARG;
        ctx->ens_graphs = value;
        return HT3D_OK;
    }
    if (key == HT3D_TUNE_TEMPORAL) {
        if (value < 0 || value > 4096) return HT3D_ERR_ARG;
        ctx->mixed_temporal = value;
        return HT3D_OK;
    }
    if (key == HT3D_TUNE_WAIT_TEST) {
        if (value < 0 || value > 1 << 20) return HT3D_ERR_ARG;
        ctx->wait_test = value;
        return HT3D_OK;
    }
    if (key == HT3D_TUNE_TIME_INNER) {
        if (value != 0 && value != 1) return HT3D_ERR_ARG;
        ctx->time_inner = value;
        return HT3D_OK;
    }
    return HT3D_ERR_ARG;
}

int ht3d_ctx_inner_timing(ht3d_ctx* ctx, double* ms, unsigned long long* launches, int reset) {
    if (!ctx) return HT3D_ERR_ARG;
    if (ms) *ms = ctx->inner_ms;
    if (launches) *launches = ctx->inner_launches;
    if (reset) {
        ctx->inner_ms = 0.0;
        ctx->inner_launches = 0;
    }
    return HT3D_OK;
}

int ht3d_ctx_synchronize(ht3d_ctx* ctx) {
    return ht3d_guard(ctx, [&]() {
        HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
        return HT3D_OK;
    }, false);
}

unsigned long long ht3d_ctx_launch_count(const ht3d_ctx* ctx) { return ctx ? ctx->launches : 0ULL; }
const char* ht3d_ctx_last_error(const ht3d_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null ctx"; }

int ht3d_sizeof_dyrel_params(void) { return (int)sizeof(ht3d_dyrel_params); }
int ht3d_sizeof_dyrel_stats(void) { return (int)sizeof(ht3d_dyrel_stats); }
int ht3d_sizeof_hrl_params(void) { return (int)sizeof(ht3d_hrl_params); }
int ht3d_sizeof_instance(void) { return (int)sizeof(ht3d_instance); }

int ht3d_reduce(ht3d_ctx* ctx, const double* a, long long n, int op, double* out) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(a && out && n > 0, "ht3d_reduce: null pointer or empty array");
        HT3D_REQUIRE(op >= 0 && op <= 4, "ht3d_reduce: unknown op");
        *out = ht3d_reduce_device(ctx, a, n, op, nullptr);
        return HT3D_OK;
    });
}

}  // extern "C"
