// Shared helpers of the dm_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dm_gb300.h"

namespace dmg {

// Kernels launched by this library since load (dm_kernel_launch_count()).
void count_launch(int k = 1);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t pow4(int e) { return int64_t(1) << (2 * e); }

// Stride (in coefficients) of qubit q's Pauli axis in an n-qubit state.
inline int64_t axis_stride(int n, int q) { return pow4(n - 1 - q); }

inline size_t dtype_size(int dtype) { return dtype == DM_F64 ? 8 : 4; }

inline bool valid_dtype(int dtype) { return dtype == DM_F64 || dtype == DM_F32; }

inline bool valid_n(int n) { return n >= 1 && n <= DM_MAX_QUBITS; }

// Number of SMs of the current device (cached per device).
int sm_count();

// Raise func's dynamic shared-memory limit to `bytes` on the current device
// (once per kernel and device; the attribute is per device).
cudaError_t ensure_max_dynamic_smem(const void *func, int bytes);

// Check the launch that was just enqueued.
inline int launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? DM_OK : DM_ERR_CUDA;
}

// Grid size for a grid-stride loop over `work` items with `threads` per block.
inline int grid_for(int64_t work, int threads, int blocks_per_sm = 8) {
    int64_t want = (work + threads - 1) / threads;
    int64_t cap = int64_t(sm_count()) * blocks_per_sm;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    return int(want);
}

}  // namespace dmg

#define DM_CHECK_ARG(cond)              \
    do {                                \
        if (!(cond)) return DM_ERR_ARG; \
    } while (0)

#define DM_CUDA_TRY(call)                                  \
    do {                                                   \
        if ((call) != cudaSuccess) {                       \
            (void)cudaGetLastError();                      \
            return DM_ERR_CUDA;                            \
        }                                                  \
    } while (0)
