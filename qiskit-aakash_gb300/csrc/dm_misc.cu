// Library-wide bookkeeping: launch counter, SM count cache, error strings.
#include <algorithm>
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

// Tile-pattern copy probe: reads and writes an FP32 state in place, tile by tile
// (tiles of 7 resident qubit axes, as the fused passes stream them), with
// 16-byte accesses and no arithmetic beyond a multiply by 1, so its rate is
// the DRAM rate that tile shape allows.  One CTA per tile at a time; chunk c
// of a tile (tile bits 2-13) sits at the XOR of its bits' element offsets.
struct TileProbe {
    int m;                               // non-resident qubits
    int64_t off[12];                     // element offset of tile bits 2..13
    int64_t nonres[DM_MAX_QUBITS];       // element stride of non-resident digit u (increasing position)
    int64_t ntiles;
};

__global__ void __launch_bounds__(256) tile_copy_probe(float *st, const __grid_constant__ TileProbe p, float one) {
    const int tid = threadIdx.x;
    for (int64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        int64_t base = 0, tt = t;
        for (int u = 0; u < p.m; ++u) {
            base += (tt & 3) * p.nonres[u];
            tt >>= 2;
        }
        float4 v[16];
        int64_t o[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int c = tid + 256 * k;
            int64_t off = 0;
#pragma unroll
            for (int b = 0; b < 12; ++b)
                if ((c >> b) & 1) off += p.off[b];
            o[k] = base + off;
            v[k] = *reinterpret_cast<const float4 *>(st + o[k]);
        }
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const float4 w = v[k];
            *reinterpret_cast<float4 *>(st + o[k]) = make_float4(w.x * one, w.y * one, w.z * one, w.w * one);
        }
    }
}

}  // namespace dmg

extern "C" int dm_tile_copy_probe(float *state_dev, int n, const int32_t *axes, void *stream) {
    if (!state_dev || !axes || n < 7 || n > DM_MAX_QUBITS || (reinterpret_cast<uintptr_t>(state_dev) & 15))
        return DM_ERR_ARG;
    if (axes[0] != n - 1) return DM_ERR_ARG;   // 16-byte chunks: the lowest axis is resident
    dmg::TileProbe p{};
    bool res[DM_MAX_QUBITS] = {false};
    for (int r = 0; r < 7; ++r) {
        if (axes[r] < 0 || axes[r] >= n || (r > 0 && axes[r] >= axes[r - 1])) return DM_ERR_ARG;
        res[axes[r]] = true;
        const int pos = n - 1 - axes[r];
        if (r > 0) {
            p.off[2 * r - 2] = int64_t(1) << (2 * pos);
            p.off[2 * r - 1] = int64_t(2) << (2 * pos);
        }
    }
    p.m = n - 7;
    int m = 0;
    for (int q = n - 1; q >= 0; --q)
        if (!res[q]) p.nonres[m++] = int64_t(1) << (2 * (n - 1 - q));
    p.ntiles = int64_t(1) << (2 * p.m);
    const int64_t grid = std::min<int64_t>(int64_t(dmg::sm_count()) * 8, p.ntiles);
    dmg::tile_copy_probe<<<int(grid), 256, 0, dmg::as_stream(stream)>>>(state_dev, p, 1.0f);
    dmg::count_launch();
    return dmg::launch_status();
}

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
