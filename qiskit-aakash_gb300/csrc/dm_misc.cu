// Library-wide bookkeeping: launch counter, SM count cache, error strings.
#include <atomic>
#include <mutex>
#include <vector>

#include "dm_common.cuh"

namespace dmg {

static std::atomic<uint64_t> g_launches{0};

void count_launch(int k) { g_launches.fetch_add(uint64_t(k), std::memory_order_relaxed); }

int sm_count() {
    static std::mutex mu;
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    std::lock_guard<std::mutex> lock(mu);
    if (cache[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
            v = 152;
        cache[dev] = v;
    }
    return cache[dev];
}

cudaError_t ensure_max_dynamic_smem(const void *func, int bytes) {
    struct Done {
        const void *func;
        int device, bytes;
    };
    static std::mutex mu;
    static std::vector<Done> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return cudaErrorInvalidDevice;
    }
    std::lock_guard<std::mutex> lock(mu);
    for (const Done &d : done)
        if (d.func == func && d.device == dev && d.bytes >= bytes) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return e;
    }
    done.push_back(Done{func, dev, bytes});
    return cudaSuccess;
}

// FP64 FMA throughput probe: every thread runs kChains independent FMA chains
// of `iters` steps (x = x * a + b, a slightly below 1 so nothing overflows)
// and writes their sum, so no FMA can be dropped.
constexpr int kFmaChains = 8;

__global__ void __launch_bounds__(256) fp64_fma_probe(double *out, int64_t iters, double a, double b) {
    double x[kFmaChains];
#pragma unroll
    for (int c = 0; c < kFmaChains; ++c) x[c] = double(threadIdx.x + c);
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kFmaChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kFmaChains; ++c) s += x[c];
    out[blockIdx.x * int64_t(blockDim.x) + threadIdx.x] = s;
}

}  // namespace dmg

extern "C" int dm_fp64_fma_probe_threads(void) { return dmg::sm_count() * 8 * 256; }

extern "C" int dm_fp64_fma_probe(double *out_dev, int64_t iters, void *stream) {
    if (!out_dev || iters < 1) return DM_ERR_ARG;
    const int blocks = dmg::sm_count() * 8;
    dmg::fp64_fma_probe<<<blocks, 256, 0, dmg::as_stream(stream)>>>(out_dev, iters, 0.999999, 1e-7);
    dmg::count_launch();
    return dmg::launch_status();
}

extern "C" const char *dm_error_string(int code) {
    switch (code) {
        case DM_OK: return "ok";
        case DM_ERR_ARG: return "invalid argument";
        case DM_ERR_CUDA: return "CUDA runtime error";
        case DM_ERR_RANGE: return "size beyond a documented limit";
        case DM_ERR_PROGRAM: return "malformed fused-pass program";
        default: return "unknown error";
    }
}

extern "C" uint64_t dm_kernel_launch_count(void) { return dmg::g_launches.load(); }

extern "C" const char *dm_version(void) { return "dm_gb300 1.0 sm_103a"; }
