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

}  // namespace dmg

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
