// State set-up, read-out and conversion kernels.
#include <math.h>
#include <string.h>

#include <vector>

#include "dm_common.cuh"

namespace dmg {

// ---------------------------------------------------------------------------
// product states (dm_simulator.py:284-349)
// ---------------------------------------------------------------------------

struct ProductSupport {
    int n;
    int nnz[DM_MAX_QUBITS];
    int8_t digit[DM_MAX_QUBITS][4];
    double val[DM_MAX_QUBITS][4];
    double scale;
};

// Writes the non-zero entries of a Kronecker product of per-qubit
// 4-vectors; the rest of the state was cleared with cudaMemsetAsync.
template <typename T>
__global__ void __launch_bounds__(256) product_kernel(T *__restrict__ st, const __grid_constant__ ProductSupport p,
                                                      int64_t support) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < support;
         i += int64_t(gridDim.x) * blockDim.x) {
        int64_t rem = i, idx = 0, stride = 1;
        double v = p.scale;
        for (int q = p.n - 1; q >= 0; --q) {
            const int k = p.nnz[q];
            const int c = int(rem % k);
            rem /= k;
            idx += int64_t(p.digit[q][c]) * stride;
            v *= p.val[q][c];
            stride <<= 2;
        }
        st[idx] = T(v);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) chop_kernel(const T *__restrict__ st, int64_t total, double thr,
                                                   double *__restrict__ out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total;
         i += int64_t(gridDim.x) * blockDim.x) {
        const double v = double(st[i]);
        out[i] = fabs(v) < thr ? 0.0 : v;
    }
}

// The same over pairs: 16-byte stores (out may be mapped host memory, written over the
// CPU-GPU link), total even, both pointers 16-byte aligned.
template <typename T>
__global__ void __launch_bounds__(256) chop_pairs_kernel(const T *__restrict__ st, int64_t pairs, double thr,
                                                         double2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < pairs;
         i += int64_t(gridDim.x) * blockDim.x) {
        const double a = double(st[2 * i]), b = double(st[2 * i + 1]);
        out[i] = make_double2(fabs(a) < thr ? 0.0 : a, fabs(b) < thr ? 0.0 : b);
    }
}

struct GatherIdx {
    int64_t idx[64];
};

template <typename T>
__global__ void gather_kernel(const T *__restrict__ st, const __grid_constant__ GatherIdx g, int count,
                              double *__restrict__ out) {
    const int i = threadIdx.x;
    if (i < count) out[i] = double(st[g.idx[i]]);
}

// ---------------------------------------------------------------------------
// overlap (dm_simulator.py:1277-1282)
// ---------------------------------------------------------------------------

constexpr int kOverlapMaxBlocks = 4096;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ double block_sum(double v) {
    __shared__ double part[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) part[w] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = threadIdx.x < nw ? part[threadIdx.x] : 0.0;
    if (w == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}

template <typename T>
__global__ void __launch_bounds__(256) dot_partial_kernel(const T *__restrict__ a, const T *__restrict__ b,
                                                          int64_t total, double *__restrict__ partial) {
    double acc = 0.0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total;
         i += int64_t(gridDim.x) * blockDim.x)
        acc = fma(double(a[i]), double(b[i]), acc);
    acc = block_sum(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(256) sum_partials_kernel(const double *__restrict__ partial, int count,
                                                           double scale, double *__restrict__ out) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) acc += partial[i];
    acc = block_sum(acc);
    if (threadIdx.x == 0) out[0] = acc * scale;
}

// max |a - b| over two states (any dtypes), in FP64: one atomicMax per block on
// the bit pattern, which orders non-negative doubles like their values.
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) max_abs_diff_kernel(const TA *__restrict__ a, const TB *__restrict__ b,
                                                           int64_t total, unsigned long long *__restrict__ out) {
    double m = 0.0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total;
         i += int64_t(gridDim.x) * blockDim.x)
        m = fmax(m, fabs(double(a[i]) - double(b[i])));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double part[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) part[w] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < int(blockDim.x >> 5); ++i) m = fmax(m, part[i]);
        atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(m)));
    }
}

// ---------------------------------------------------------------------------
// Pauli basis -> matrix basis (dm_simulator.py:1198-1255)
// Per axis (I,X,Y,Z) -> (e00,e01,e10,e11) = (I+Z, X-iY, X+iY, I-Z); then the
// (row bit, column bit) pairs of every qubit are de-interleaved.
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(256) to_complex_last_axis(const T *__restrict__ st, int64_t groups,
                                                            double2 *__restrict__ buf) {
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < groups;
         g += int64_t(gridDim.x) * blockDim.x) {
        const double I = double(st[4 * g]), X = double(st[4 * g + 1]);
        const double Y = double(st[4 * g + 2]), Z = double(st[4 * g + 3]);
        buf[4 * g] = make_double2(I + Z, 0.0);
        buf[4 * g + 1] = make_double2(X, -Y);
        buf[4 * g + 2] = make_double2(X, Y);
        buf[4 * g + 3] = make_double2(I - Z, 0.0);
    }
}

__global__ void __launch_bounds__(256) to_matrix_axis(double2 *__restrict__ buf, int log4s, int64_t groups) {
    const int64_t s = int64_t(1) << (2 * log4s);
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < groups;
         g += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i0 = ((g >> (2 * log4s)) << (2 * log4s + 2)) | (g & (s - 1));
        const double2 I = buf[i0], X = buf[i0 + s], Y = buf[i0 + 2 * s], Z = buf[i0 + 3 * s];
        buf[i0] = make_double2(I.x + Z.x, I.y + Z.y);
        buf[i0 + s] = make_double2(X.x + Y.y, X.y - Y.x);       // X - iY
        buf[i0 + 2 * s] = make_double2(X.x - Y.y, X.y + Y.x);   // X + iY
        buf[i0 + 3 * s] = make_double2(I.x - Z.x, I.y - Z.y);
    }
}

__global__ void __launch_bounds__(256) deinterleave_kernel(const double2 *__restrict__ buf, int n,
                                                           double2 *__restrict__ out) {
    const int64_t dim = int64_t(1) << n, total = dim * dim;
    for (int64_t o = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; o < total;
         o += int64_t(gridDim.x) * blockDim.x) {
        const int64_t r = o >> n, c = o & (dim - 1);
        int64_t idx = 0;
        for (int j = 0; j < n; ++j) idx |= (((r >> j) & 1) << (2 * j + 1)) | (((c >> j) & 1) << (2 * j));
        out[o] = buf[idx];
    }
}

}  // namespace dmg

using namespace dmg;

extern "C" int dm_init_product(void *state_dev, int n, int dtype, const double *v, double scale, void *stream) {
    DM_CHECK_ARG(state_dev && v && valid_n(n) && valid_dtype(dtype));
    ProductSupport p;
    memset(&p, 0, sizeof(p));
    p.n = n;
    p.scale = scale;
    int64_t support = 1;
    for (int q = 0; q < n; ++q) {
        int k = 0;
        for (int d = 0; d < 4; ++d)
            if (v[4 * q + d] != 0.0) {
                p.digit[q][k] = int8_t(d);
                p.val[q][k] = v[4 * q + d];
                ++k;
            }
        if (k == 0) {  // an all-zero factor: the whole state is zero
            p.nnz[q] = 1;
            p.digit[q][0] = 0;
            p.val[q][0] = 0.0;
            k = 1;
        }
        p.nnz[q] = k;
        support *= k;
    }
    cudaStream_t s = as_stream(stream);
    DM_CUDA_TRY(cudaMemsetAsync(state_dev, 0, size_t(pow4(n)) * dtype_size(dtype), s));
    if (dtype == DM_F64)
        product_kernel<double><<<grid_for(support, 256), 256, 0, s>>>(static_cast<double *>(state_dev), p, support);
    else
        product_kernel<float><<<grid_for(support, 256), 256, 0, s>>>(static_cast<float *>(state_dev), p, support);
    count_launch();
    return launch_status();
}

extern "C" int dm_load_state(void *state_dev, int n, int dtype, const double *host_coeffs, void *stream) {
    DM_CHECK_ARG(state_dev && host_coeffs && valid_n(n) && valid_dtype(dtype));
    const size_t total = size_t(pow4(n));
    cudaStream_t s = as_stream(stream);
    if (dtype == DM_F64) {
        DM_CUDA_TRY(cudaMemcpyAsync(state_dev, host_coeffs, total * 8, cudaMemcpyHostToDevice, s));
        DM_CUDA_TRY(cudaStreamSynchronize(s));
        return DM_OK;
    }
    std::vector<float> tmp(total);
    for (size_t i = 0; i < total; ++i) tmp[i] = float(host_coeffs[i]);
    DM_CUDA_TRY(cudaMemcpyAsync(state_dev, tmp.data(), total * 4, cudaMemcpyHostToDevice, s));
    DM_CUDA_TRY(cudaStreamSynchronize(s));
    return DM_OK;
}

extern "C" int dm_chop_copy(const void *state_dev, int n, int dtype, double threshold, double *out_dev,
                            void *stream) {
    DM_CHECK_ARG(valid_n(n));
    return dm_chop_copy_range(state_dev, n, dtype, 0, pow4(n), threshold, out_dev, stream);
}

extern "C" int dm_chop_copy_range(const void *state_dev, int n, int dtype, int64_t offset, int64_t count,
                                  double threshold, double *out_dev, void *stream) {
    DM_CHECK_ARG(state_dev && out_dev && valid_n(n) && valid_dtype(dtype));
    DM_CHECK_ARG(offset >= 0 && count > 0 && offset + count <= pow4(n));
    const int64_t total = count;
    if (dtype == DM_F64)
        state_dev = static_cast<const double *>(state_dev) + offset;
    else
        state_dev = static_cast<const float *>(state_dev) + offset;
    cudaStream_t s = as_stream(stream);
    if (total % 2 == 0 && (reinterpret_cast<uintptr_t>(out_dev) & 15) == 0) {
        const int64_t pairs = total / 2;
        auto *out2 = reinterpret_cast<double2 *>(out_dev);
        if (dtype == DM_F64)
            chop_pairs_kernel<double><<<grid_for(pairs, 256), 256, 0, s>>>(static_cast<const double *>(state_dev),
                                                                          pairs, threshold, out2);
        else
            chop_pairs_kernel<float><<<grid_for(pairs, 256), 256, 0, s>>>(static_cast<const float *>(state_dev),
                                                                         pairs, threshold, out2);
    } else if (dtype == DM_F64) {
        chop_kernel<double><<<grid_for(total, 256), 256, 0, s>>>(static_cast<const double *>(state_dev), total,
                                                                 threshold, out_dev);
    } else {
        chop_kernel<float><<<grid_for(total, 256), 256, 0, s>>>(static_cast<const float *>(state_dev), total,
                                                                threshold, out_dev);
    }
    count_launch();
    return launch_status();
}

extern "C" void *dm_host_alloc(size_t bytes) {
    if (bytes == 0) return nullptr;
    void *p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return p;
}

extern "C" void *dm_host_device_pointer(void *host) {
    void *d = nullptr;
    if (!host || cudaHostGetDevicePointer(&d, host, 0) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return d;
}

extern "C" int dm_host_free(void *host) {
    if (!host) return DM_ERR_ARG;
    DM_CUDA_TRY(cudaFreeHost(host));
    return DM_OK;
}

extern "C" int dm_gather(const void *state_dev, int n, int dtype, const int64_t *idx, int count, double *out_dev,
                         void *stream) {
    DM_CHECK_ARG(state_dev && idx && out_dev && valid_n(n) && valid_dtype(dtype));
    DM_CHECK_ARG(count >= 1 && count <= 64);
    GatherIdx g;
    const int64_t total = pow4(n);
    for (int i = 0; i < count; ++i) {
        DM_CHECK_ARG(idx[i] >= 0 && idx[i] < total);
        g.idx[i] = idx[i];
    }
    cudaStream_t s = as_stream(stream);
    if (dtype == DM_F64)
        gather_kernel<double><<<1, 64, 0, s>>>(static_cast<const double *>(state_dev), g, count, out_dev);
    else
        gather_kernel<float><<<1, 64, 0, s>>>(static_cast<const float *>(state_dev), g, count, out_dev);
    count_launch();
    return launch_status();
}

extern "C" size_t dm_overlap_scratch_bytes(int n) {
    (void)n;
    return sizeof(double) * kOverlapMaxBlocks;
}

extern "C" int dm_overlap(const void *a_dev, const void *b_dev, int n, int dtype, double *out_dev, void *scratch_dev,
                          void *stream) {
    DM_CHECK_ARG(a_dev && b_dev && out_dev && scratch_dev && valid_n(n) && valid_dtype(dtype));
    const int64_t total = pow4(n);
    int blocks = grid_for(total, 256, 4);
    if (blocks > kOverlapMaxBlocks) blocks = kOverlapMaxBlocks;
    cudaStream_t s = as_stream(stream);
    double *partial = static_cast<double *>(scratch_dev);
    if (dtype == DM_F64)
        dot_partial_kernel<double><<<blocks, 256, 0, s>>>(static_cast<const double *>(a_dev),
                                                          static_cast<const double *>(b_dev), total, partial);
    else
        dot_partial_kernel<float><<<blocks, 256, 0, s>>>(static_cast<const float *>(a_dev),
                                                         static_cast<const float *>(b_dev), total, partial);
    count_launch();
    int rc = launch_status();
    if (rc) return rc;
    sum_partials_kernel<<<1, 256, 0, s>>>(partial, blocks, ldexp(1.0, n), out_dev);
    count_launch();
    return launch_status();
}

extern "C" size_t dm_pauli_to_matrix_scratch_bytes(int n) {
    if (!valid_n(n)) return 0;
    return size_t(pow4(n)) * sizeof(double2);
}

extern "C" int dm_pauli_to_matrix(const void *state_dev, int n, int dtype, double *out_dev, void *scratch_dev,
                                  void *stream) {
    DM_CHECK_ARG(state_dev && out_dev && scratch_dev && valid_n(n) && valid_dtype(dtype));
    if (n > 15) return DM_ERR_RANGE;  // 2**n x 2**n complex128 output beyond 16 GB
    cudaStream_t s = as_stream(stream);
    double2 *buf = static_cast<double2 *>(scratch_dev);
    const int64_t groups = pow4(n - 1);
    if (dtype == DM_F64)
        to_complex_last_axis<double><<<grid_for(groups, 256), 256, 0, s>>>(static_cast<const double *>(state_dev),
                                                                            groups, buf);
    else
        to_complex_last_axis<float><<<grid_for(groups, 256), 256, 0, s>>>(static_cast<const float *>(state_dev),
                                                                           groups, buf);
    count_launch();
    int rc = launch_status();
    if (rc) return rc;
    for (int q = n - 2; q >= 0; --q) {
        to_matrix_axis<<<grid_for(groups, 256), 256, 0, s>>>(buf, n - 1 - q, groups);
        count_launch();
        if ((rc = launch_status())) return rc;
    }
    const int64_t total = pow4(n);
    deinterleave_kernel<<<grid_for(total, 256), 256, 0, s>>>(buf, n, reinterpret_cast<double2 *>(out_dev));
    count_launch();
    return launch_status();
}

extern "C" int dm_max_abs_diff(const void *a_dev, int dtype_a, const void *b_dev, int dtype_b, int n, double *out_dev,
                               void *stream) {
    DM_CHECK_ARG(a_dev && b_dev && out_dev && valid_n(n) && valid_dtype(dtype_a) && valid_dtype(dtype_b));
    const int64_t total = pow4(n);
    cudaStream_t s = as_stream(stream);
    DM_CUDA_TRY(cudaMemsetAsync(out_dev, 0, sizeof(double), s));
    const int blocks = grid_for(total, 256, 4);
    auto *out = reinterpret_cast<unsigned long long *>(out_dev);
    if (dtype_a == DM_F32 && dtype_b == DM_F64)
        max_abs_diff_kernel<<<blocks, 256, 0, s>>>(static_cast<const float *>(a_dev), static_cast<const double *>(b_dev),
                                                   total, out);
    else if (dtype_a == DM_F64 && dtype_b == DM_F64)
        max_abs_diff_kernel<<<blocks, 256, 0, s>>>(static_cast<const double *>(a_dev),
                                                   static_cast<const double *>(b_dev), total, out);
    else if (dtype_a == DM_F32 && dtype_b == DM_F32)
        max_abs_diff_kernel<<<blocks, 256, 0, s>>>(static_cast<const float *>(a_dev), static_cast<const float *>(b_dev),
                                                   total, out);
    else
        max_abs_diff_kernel<<<blocks, 256, 0, s>>>(static_cast<const double *>(a_dev),
                                                   static_cast<const float *>(b_dev), total, out);
    count_launch();
    return launch_status();
}
