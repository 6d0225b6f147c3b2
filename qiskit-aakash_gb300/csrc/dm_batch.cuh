// Instance set-up and read-out of the batched sweeps (persistent CTAs of NT
// threads, one instance at a time).
#pragma once

#include "dm_common.cuh"

namespace dmg {

// |0...0>: a = 2**-n on the {I, Z}**n sub-lattice, 0 elsewhere.  Called by all threads.
template <typename T, int NT>
__device__ void batch_init_zero(T *st, int n) {
    const int tid = threadIdx.x;
    const int64_t total = int64_t(1) << (2 * n);
    for (int64_t e = int64_t(tid) * 4; e < total; e += 4 * NT) {
        st[e] = T(0);
        st[e + 1] = T(0);
        st[e + 2] = T(0);
        st[e + 3] = T(0);
    }
    __syncthreads();
    const T amp = T(ldexp(1.0, -n));
    for (int i = tid; i < (1 << n); i += NT) {
        int64_t idx = 0;
        for (int q = 0; q < n; ++q)
            if ((i >> q) & 1) idx += int64_t(3) << (2 * q);
        st[idx] = amp;
    }
    __syncthreads();
}

// Z read-out: gather the 2**n sub-lattice coefficients, scale by err**popcount,
// Walsh-Hadamard transform in shared memory (outcome bit of qubit 0 is the MSB).
template <typename T, int NT>
__device__ void batch_z_readout(const T *st, int n, double err, double *out, double *wv) {
    const int tid = threadIdx.x;
    const int np = 1 << n;
    for (int i = tid; i < np; i += NT) {
        int64_t idx = 0;
        double w = 1.0;
        for (int j = 0; j < n; ++j)
            if ((i >> (n - 1 - j)) & 1) {
                idx += int64_t(3) << (2 * (n - 1 - j));
                w *= err;
            }
        wv[i] = double(st[idx]) * w;
    }
    __syncthreads();
    for (int b = 0; b < n; ++b) {
        for (int pidx = tid; pidx < np / 2; pidx += NT) {
            const int i0 = ((pidx >> b) << (b + 1)) | (pidx & ((1 << b) - 1));
            const int i1 = i0 | (1 << b);
            const double x = wv[i0], y = wv[i1];
            wv[i0] = x + y;
            wv[i1] = x - y;
        }
        __syncthreads();
    }
    for (int i = tid; i < np; i += NT) out[i] = wv[i];
    __syncthreads();
}

}  // namespace dmg
