// Measurement probabilities (dm_simulator.py:427-538).
//
// For measurement axis col_q (1=X, 2=Y, 3=Z) on qubit q with polarisation
// err, the probability of outcome b is
//     P(b) = sum_{s in {0, col}^n} a_s prod_q w(s_q, b_q),
//     w(0, b) = 1,  w(col, 0) = err,  w(col, 1) = -err,
// the row-times-vector product the reference forms with a 2**n x 2**n
// Kronecker matrix (dm_simulator.py:444-468).  Here: gather the 2**m
// coefficients of the sub-lattice (unmeasured qubits pinned to I, which is
// what summing P over their outcomes leaves, times 2 each), scale by
// err**popcount and apply an in-place Walsh-Hadamard transform.
#include <math.h>

#include <cuda.h>

#include <mutex>

#include "dm_common.cuh"

namespace dmg {

struct SubLattice {
    int m;
    int64_t stride[DM_MAX_QUBITS];   // flat-index step of measured bit j (bit m-1-j of the outcome)
    double errpow[DM_MAX_QUBITS + 1];
    double scale;                    // 2**(n-m)
};

template <typename T>
__global__ void __launch_bounds__(256) sublattice_gather(const T *__restrict__ st, const __grid_constant__ SubLattice L,
                                                         double *__restrict__ out) {
    const int64_t total = int64_t(1) << L.m;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total;
         i += int64_t(gridDim.x) * blockDim.x) {
        int64_t idx = 0;
        int pop = 0;
        for (int j = 0; j < L.m; ++j)
            if ((i >> (L.m - 1 - j)) & 1) {
                idx += L.stride[j];
                ++pop;
            }
        out[i] = double(st[idx]) * L.errpow[pop] * L.scale;
    }
}

// In-place unnormalised Walsh-Hadamard butterflies over bits [lo, lo+nb) of
// a 2**m vector; each CTA transforms one tile of 2**nb elements in shared
// memory.
constexpr int kWhtTileBits = 11;

__global__ void __launch_bounds__(256) wht_kernel(double *__restrict__ v, int m, int lo, int nb) {
    __shared__ double tile[1 << kWhtTileBits];
    const int tsize = 1 << nb;
    const int64_t ntiles = int64_t(1) << (m - nb);
    const int64_t lomask = (int64_t(1) << lo) - 1;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t base = (t & lomask) | ((t >> lo) << (lo + nb));
        for (int e = threadIdx.x; e < tsize; e += blockDim.x) tile[e] = v[base | (int64_t(e) << lo)];
        __syncthreads();
        for (int b = 0; b < nb; ++b) {
            for (int p = threadIdx.x; p < tsize / 2; p += blockDim.x) {
                const int i0 = ((p >> b) << (b + 1)) | (p & ((1 << b) - 1));
                const int i1 = i0 | (1 << b);
                const double x = tile[i0], y = tile[i1];
                tile[i0] = x + y;
                tile[i1] = x - y;
            }
            __syncthreads();
        }
        for (int e = threadIdx.x; e < tsize; e += blockDim.x) v[base | (int64_t(e) << lo)] = tile[e];
        __syncthreads();
    }
}

static int wht_inplace(double *v, int m, cudaStream_t s) {
    for (int lo = 0; lo < m; lo += kWhtTileBits) {
        const int nb = (m - lo) < kWhtTileBits ? (m - lo) : kWhtTileBits;
        const int64_t ntiles = int64_t(1) << (m - nb);
        const int grid = int(ntiles < int64_t(sm_count()) * 4 ? ntiles : int64_t(sm_count()) * 4);
        wht_kernel<<<grid, 256, 0, s>>>(v, m, lo, nb);
        count_launch();
        int rc = launch_status();
        if (rc) return rc;
    }
    return DM_OK;
}

// --- basis N: contraction of every axis with the rows [1, +-err n] ----------

struct NRows {
    double w[2][4];
};

// Contract the lowest t axes (contiguous 4**t block per thread) into 2**t values.
template <typename T>
__global__ void __launch_bounds__(256) contract_low(const T *__restrict__ st, int t, int64_t outer,
                                                    const __grid_constant__ NRows R, double *__restrict__ out) {
    const int blk = 1 << (2 * t);
    for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < outer;
         o += int64_t(gridDim.x) * blockDim.x) {
        double v[64];
        for (int e = 0; e < blk; ++e) v[e] = double(st[o * blk + e]);
        // contract axes from the fastest: shape (4^(t-j), 2^j) -> (4^(t-j-1), 2^(j+1))
        int rows4 = blk >> 2;   // number of 4-groups on the current fastest 4-axis
        int inner = 1;          // 2^j
        for (int j = 0; j < t; ++j) {
            // current layout: index = (h * 4 + p) * inner + i, h < rows4/inner... use a temp
            double w[64];
            const int outer_h = rows4 / inner;
            for (int h = 0; h < outer_h; ++h)
                for (int i = 0; i < inner; ++i) {
                    double acc0 = 0.0, acc1 = 0.0;
                    for (int p = 0; p < 4; ++p) {
                        const double x = v[(h * 4 + p) * inner + i];
                        acc0 = fma(R.w[0][p], x, acc0);
                        acc1 = fma(R.w[1][p], x, acc1);
                    }
                    w[(h * 2 + 0) * inner + i] = acc0;
                    w[(h * 2 + 1) * inner + i] = acc1;
                }
            inner *= 2;
            rows4 /= 2;
            const int cnt = outer_h * 2 * (inner / 2);
            for (int e = 0; e < cnt; ++e) v[e] = w[e];
        }
        const int nout = 1 << t;
        for (int e = 0; e < nout; ++e) out[o * nout + e] = v[e];
    }
}

// (outer, 4, inner) -> (outer, 2, inner)
__global__ void __launch_bounds__(256) contract_axis(const double *__restrict__ in, int64_t outer, int64_t inner,
                                                     const __grid_constant__ NRows R, double *__restrict__ out) {
    const int64_t total = outer * inner;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total;
         g += int64_t(gridDim.x) * blockDim.x) {
        const int64_t o = g / inner, i = g - o * inner;
        const double *src = in + o * 4 * inner + i;
        double acc0 = 0.0, acc1 = 0.0;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const double x = src[p * inner];
            acc0 = fma(R.w[0][p], x, acc0);
            acc1 = fma(R.w[1][p], x, acc1);
        }
        out[o * 2 * inner + i] = acc0;
        out[o * 2 * inner + inner + i] = acc1;
    }
}

}  // namespace dmg

using namespace dmg;

extern "C" int dm_axis_probs(const void *state_dev, int n, int dtype, const int *mode, double err, double *out_dev,
                             void *stream) {
    DM_CHECK_ARG(state_dev && mode && out_dev && valid_n(n) && valid_dtype(dtype));
    SubLattice L;
    L.m = 0;
    for (int q = 0; q < n; ++q) {
        DM_CHECK_ARG(mode[q] >= 0 && mode[q] <= 3);
        if (mode[q]) L.stride[L.m++] = int64_t(mode[q]) * axis_stride(n, q);
    }
    L.errpow[0] = 1.0;
    for (int j = 1; j <= DM_MAX_QUBITS; ++j) L.errpow[j] = L.errpow[j - 1] * err;
    L.scale = ldexp(1.0, n - L.m);
    cudaStream_t s = as_stream(stream);
    const int64_t total = int64_t(1) << L.m;
    if (dtype == DM_F64)
        sublattice_gather<double><<<grid_for(total, 256), 256, 0, s>>>(static_cast<const double *>(state_dev), L,
                                                                       out_dev);
    else
        sublattice_gather<float><<<grid_for(total, 256), 256, 0, s>>>(static_cast<const float *>(state_dev), L,
                                                                      out_dev);
    count_launch();
    int rc = launch_status();
    if (rc || L.m == 0) return rc;
    return wht_inplace(out_dev, L.m, s);
}

static int low_axes(int n) { return n < 3 ? n : 3; }

extern "C" size_t dm_nbasis_probs_scratch_bytes(int n) {
    if (!valid_n(n)) return 0;
    const int t = low_axes(n);
    if (t == n) return 0;
    const size_t first = size_t(pow4(n - t)) << t;   // after contracting the low t axes
    return (first + first / 2) * sizeof(double);
}

extern "C" int dm_nbasis_probs(const void *state_dev, int n, int dtype, const double *nvec3, double err,
                               double *out_dev, void *scratch_dev, void *stream) {
    DM_CHECK_ARG(state_dev && nvec3 && out_dev && valid_n(n) && valid_dtype(dtype));
    const int t = low_axes(n);
    DM_CHECK_ARG(t == n || scratch_dev);
    NRows R;
    R.w[0][0] = R.w[1][0] = 1.0;
    for (int c = 0; c < 3; ++c) {
        R.w[0][c + 1] = err * nvec3[c];
        R.w[1][c + 1] = -err * nvec3[c];
    }
    cudaStream_t s = as_stream(stream);
    const size_t first = size_t(pow4(n - t)) << t;
    double *bufA = static_cast<double *>(scratch_dev);
    double *bufB = bufA ? bufA + first : nullptr;
    double *dst = (t == n) ? out_dev : bufA;
    const int64_t outer = pow4(n - t);
    if (dtype == DM_F64)
        contract_low<double><<<grid_for(outer, 256), 256, 0, s>>>(static_cast<const double *>(state_dev), t, outer,
                                                                  R, dst);
    else
        contract_low<float><<<grid_for(outer, 256), 256, 0, s>>>(static_cast<const float *>(state_dev), t, outer, R,
                                                                 dst);
    count_launch();
    int rc = launch_status();
    if (rc || t == n) return rc;
    const double *src = bufA;
    for (int q = n - t - 1; q >= 0; --q) {
        const int64_t o = pow4(q), inner = int64_t(1) << (n - 1 - q);
        double *d = (q == 0) ? out_dev : (src == bufA ? bufB : bufA);
        contract_axis<<<grid_for(o * inner, 256), 256, 0, s>>>(src, o, inner, R, d);
        count_launch();
        if ((rc = launch_status())) return rc;
        src = d;
    }
    return DM_OK;
}

// ---------------------------------------------------------------------------
// dm_nbasis_probs_noalloc: the basis-N probabilities with the scratch held in
// a file-scope device array instead of a caller buffer.
// ---------------------------------------------------------------------------

namespace dmg {

constexpr int kNoallocMaxQubits = 10;
// Contraction buffers for n <= kNoallocMaxQubits: 4**7 * 2**3 doubles after
// the first (three-axis) step plus half that for the ping-pong partner.
constexpr size_t kNoallocScratchDoubles = (size_t(1) << 14) * 8 * 3 / 2;   // 196,608 doubles = 1.5 MiB

// Every GPU that loads this library holds this array until the process exits.
static __device__ __align__(256) double g_nbasis_scratch[kNoallocScratchDoubles];

constexpr int kMaxDevices = 64;

// The unique ID of the current CUDA context (driver entry points resolved at
// run time), or 0 when it cannot be read.  A device's primary context gets a
// new ID when it is destroyed and created again (cudaDeviceReset), and the
// module holding g_nbasis_scratch is then loaded again, possibly elsewhere.
static unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static std::once_flag once;
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(p);
        (void)cudaGetLastError();
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr ||
        get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of g_nbasis_scratch, resolved with the device current, once
// per device and context: it is looked up again when the device's context
// has changed since (or when its ID cannot be read).  Host code must not pass
// the symbol itself to a kernel: on the host it names a shadow variable, not
// device memory.
static int noalloc_scratch(double **out) {
    static std::mutex mu;
    static double *addr[kMaxDevices] = {nullptr};
    static unsigned long long ctx_of[kMaxDevices] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return DM_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) return DM_ERR_RANGE;
    // 0 (no context current on this thread yet, or no ID): look the address up, which also makes
    // the runtime's context current; a later call then records that context's ID
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lock(mu);
    if (addr[dev] == nullptr || ctx == 0 || ctx != ctx_of[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_nbasis_scratch) != cudaSuccess) {
            (void)cudaGetLastError();
            return DM_ERR_CUDA;
        }
        addr[dev] = static_cast<double *>(p);
        ctx_of[dev] = ctx;
    }
    *out = addr[dev];
    return DM_OK;
}

}  // namespace dmg

extern "C" int dm_nbasis_probs_noalloc(const void *state_dev, int n, int dtype, const double *nvec3, double err,
                                       double *out_dev, void *stream) {
    DM_CHECK_ARG(state_dev && nvec3 && out_dev && valid_n(n) && valid_dtype(dtype));
    if (n > kNoallocMaxQubits) return DM_ERR_RANGE;
    const int t = low_axes(n);
    double *scratch = nullptr;
    if (t < n) {
        int rc = noalloc_scratch(&scratch);
        if (rc) return rc;
    }
    NRows R;
    R.w[0][0] = R.w[1][0] = 1.0;
    for (int c = 0; c < 3; ++c) {
        R.w[0][c + 1] = err * nvec3[c];
        R.w[1][c + 1] = -err * nvec3[c];
    }
    cudaStream_t s = as_stream(stream);
    // Every buffer element read below is written earlier in the same call,
    // so the array's contents from a previous call never leak into a result.
    const size_t first = size_t(pow4(n - t)) << t;
    double *bufA = scratch;
    double *bufB = scratch ? scratch + first : nullptr;
    double *dst = (t == n) ? out_dev : bufA;
    const int64_t outer = pow4(n - t);
    if (dtype == DM_F64)
        contract_low<double><<<grid_for(outer, 256), 256, 0, s>>>(static_cast<const double *>(state_dev), t, outer,
                                                                  R, dst);
    else
        contract_low<float><<<grid_for(outer, 256), 256, 0, s>>>(static_cast<const float *>(state_dev), t, outer, R,
                                                                 dst);
    count_launch();
    int rc = launch_status();
    if (rc || t == n) return rc;
    const double *src = bufA;
    for (int q = n - t - 1; q >= 0; --q) {
        const int64_t o = pow4(q), inner = int64_t(1) << (n - 1 - q);
        double *d = (q == 0) ? out_dev : (src == bufA ? bufB : bufA);
        contract_axis<<<grid_for(o * inner, 256), 256, 0, s>>>(src, o, inner, R, d);
        count_launch();
        if ((rc = launch_status())) return rc;
        src = d;
    }
    return DM_OK;
}
