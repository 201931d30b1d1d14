// Library-level C ABI: version, status strings, thread-local error messages.
#include "tt_internal.cuh"

namespace tt {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

tt_status check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return TT_ERR_CUDA;
    }
    return TT_OK;
}

int sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

// FMA issue-rate probe: 8 independent dependency chains per thread, so that the FP64 (or FP32)
// pipe, not latency, sets the time.  Every thread writes its sum (nothing is dead code).
template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(int64_t iters, T a, T b, T* sink) {
    T x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = T(threadIdx.x * 1e-3 + c);
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    sink[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace tt

extern "C" {

tt_status tt_fma_probe(int64_t iters, int32_t blocks, int32_t prec, void* sink, void* stream) {
    if (iters < 0 || blocks <= 0 || !sink) {
        tt::set_error("tt_fma_probe: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (prec == TT_PREC_F32)
        tt::fma_probe_kernel<float><<<blocks, 256, 0, tt::as_stream(stream)>>>(iters, 0.9999999f, 1e-7f,
                                                                              static_cast<float*>(sink));
    else
        tt::fma_probe_kernel<double><<<blocks, 256, 0, tt::as_stream(stream)>>>(iters, 0.9999999, 1e-7,
                                                                               static_cast<double*>(sink));
    return tt::check_launch("tt_fma_probe");
}

int32_t tt_abi_version(void) { return TT_ABI_VERSION; }

const char* tt_status_string(tt_status s) {
    switch (s) {
        case TT_OK: return "ok";
        case TT_ERR_INVALID: return "invalid argument";
        case TT_ERR_NUMERIC: return "exp(Q*t) argument out of range";
        case TT_ERR_OOM: return "workspace too small";
        case TT_ERR_TIMEOUT: return "device wait timed out";
        case TT_ERR_CUDA: return "CUDA error";
        case TT_ERR_UNSUPPORTED: return "unsupported";
        case TT_ERR_BRACKET: return "Brent bracket condition not met";
        default: return "unknown status";
    }
}

size_t tt_last_error(char* buf, size_t n) {
    const std::string& s = tt::g_last_error;
    if (buf && n) {
        size_t k = s.size() < n - 1 ? s.size() : n - 1;
        memcpy(buf, s.data(), k);
        buf[k] = 0;
    }
    return s.size();
}

int32_t tt_device_sm_count(void) { return tt::sm_count(); }

}  // extern "C"
