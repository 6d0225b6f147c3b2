// Kernels of the noise-surrogate MLP ensemble (no reference counterpart).
//
// The network maps noise parameters to a fixed circuit's outcome
// distribution.  Its matrix products run on the tensor cores: one CTA of
// 128 threads computes a 128 x 64 tile of C = A B^T with BF16 operands
// (kind::f16, FP32 accumulation in 64 TMEM columns).  K is streamed in
// 64-wide chunks by cp.async into two shared-memory stages in the K-major
// core-matrix layout; one thread issues the four K = 16 MMAs of a chunk and
// commits them to an mbarrier while all threads fetch the next chunk.  The
// epilogue (one accumulator row per thread, tcgen05.ld) applies bias and
// GELU, or the GELU derivative of the backward pass, and writes the
// row-major result plus, where the next product needs it, its transpose, so
// that every later product is again of the A B^T form with K contiguous.
// Waits on the mbarrier are bounded and record an error in *status.
//
// The other kernels are memory-light helpers: softmax with the KL loss and
// its gradient, bias gradients, Adam with the BF16 weight copies, the
// minibatch gather and the ensemble statistics.
#include <cuda_bf16.h>

#include <mutex>

#include "dm_common.cuh"
#include "dm_tcgen05.cuh"

namespace dmg {
namespace mlp {

constexpr int kThreads = 128;
constexpr int kBM = 128, kBN = 64, kBK = 64;
// K-major core-matrix layout of a rows x 64 BF16 chunk: element (row, k) at
// byte (row%8)*16 + (k%8)*2 + (k/8)*128 + (row/8)*1024.
constexpr uint32_t kLBO = 128, kSBO = 1024;
constexpr uint32_t kABytes = kBM * kBK * 2;        // 16 KB
constexpr uint32_t kBBytes = kBN * kBK * 2;        // 8 KB
constexpr uint32_t kStage = kABytes + kBBytes;     // 24 KB
constexpr uint32_t kSmemBytes = 2 * kStage;        // 48 KB
constexpr uint32_t kTmemCols = 64;
// kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9 and 10-12 = 1), K-major, N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t(kBN) >> 3) << 17) |
                            ((uint32_t(kBM) >> 4) << 24);

constexpr float kGeluC = 0.7978845608028654f;   // sqrt(2 / pi)
constexpr float kGeluA = 0.044715f;

__device__ __forceinline__ float gelu(float u) {
    return 0.5f * u * (1.0f + tanhf(kGeluC * fmaf(kGeluA * u * u, u, u)));
}

__device__ __forceinline__ float gelu_grad(float u) {
    const float t = tanhf(kGeluC * fmaf(kGeluA * u * u, u, u));
    return 0.5f * (1.0f + t) + 0.5f * u * (1.0f - t * t) * kGeluC * fmaf(3.0f * kGeluA, u * u, 1.0f);
}

__device__ __forceinline__ uint16_t to_bf16(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float from_bf16(uint16_t b) { return __uint_as_float(uint32_t(b) << 16); }

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    return uint32_t(to_bf16(a)) | (uint32_t(to_bf16(b)) << 16);
}

template <int EPI>
__global__ void __launch_bounds__(kThreads) gemm_kernel(const dm_mlp_gemm g, int *status) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_s;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
    const int64_t z = blockIdx.z;
    const uint16_t *A = g.A + z * g.a_ms + int64_t(m0) * g.lda;
    const uint16_t *B = g.B + z * g.b_ms + int64_t(n0) * g.ldb;

    if (tid == 0) {
        abort_s = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tcg::smem_u32(&mbar)));
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         tcg::smem_u32(&tmem_base_s)),
                     "n"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;

    auto load_chunk = [&](int c, int s) {
        unsigned char *sa = smem + s * kStage, *sb = sa + kABytes;
        const int k0 = c * kBK;
        for (int i = tid; i < kBM * 8; i += kThreads) {       // 8 16-byte pieces per row
            const int r = i >> 3, p = i & 7;
            tcg::cp_async16(sa + (r & 7) * 16 + p * kLBO + (r >> 3) * kSBO, A + int64_t(r) * g.lda + k0 + 8 * p);
        }
        for (int i = tid; i < kBN * 8; i += kThreads) {
            const int r = i >> 3, p = i & 7;
            tcg::cp_async16(sb + (r & 7) * 16 + p * kLBO + (r >> 3) * kSBO, B + int64_t(r) * g.ldb + k0 + 8 * p);
        }
        tcg::cp_async_commit();
    };

    const int nch = g.K / kBK;
    uint32_t phase = 0;
    bool pending = false;     // an MMA batch is committed but not yet waited for
    load_chunk(0, 0);
    for (int c = 0; c < nch; ++c) {
        tcg::cp_async_wait_all();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
            const uint32_t a = tcg::smem_u32(smem + (c & 1) * kStage), b = a + kABytes;
#pragma unroll
            for (int ks = 0; ks < kBK / 16; ++ks) {
                const uint64_t da = tcg::smem_desc(a + ks * 2 * kLBO, kLBO, kSBO);
                const uint64_t db = tcg::smem_desc(b + ks * 2 * kLBO, kLBO, kSBO);
                const uint32_t acc = (c | ks) ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(kIdesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                tcg::smem_u32(&mbar)));
        }
        pending = true;
        // the other stage was read by the previous chunk's MMAs, which have completed
        if (c + 1 < nch) load_chunk(c + 1, (c + 1) & 1);
        const bool ok = tcg::mbar_wait(tcg::smem_u32(&mbar), phase);
        if (ok) {
            phase ^= 1;
            pending = false;
        }
        if (!__all_sync(0xffffffffu, ok) && (tid & 31) == 0) {
            atomicExch(status, 1);
            abort_s = 1;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        __syncthreads();
        if (abort_s) break;
    }

    if (!abort_s) {
        float v[64];
        tcg::tmem_ld64(tmem + (uint32_t(32 * warp) << 16), v);
        const int64_t row = m0 + tid;
        if constexpr (EPI == DM_MLP_EPI_GELU_FWD || EPI == DM_MLP_EPI_BIAS_F32) {
            const float *bias = g.bias + z * g.bias_ms + n0;
#pragma unroll
            for (int j = 0; j < 64; ++j) v[j] += bias[j];
        }
        if constexpr (EPI == DM_MLP_EPI_GELU_FWD || EPI == DM_MLP_EPI_BIAS_F32 || EPI == DM_MLP_EPI_F32) {
            if (g.out_f32) {
                float *o = g.out_f32 + z * g.f32_ms + row * g.ld_f32 + n0;
#pragma unroll
                for (int j = 0; j < 64; j += 4) *reinterpret_cast<float4 *>(o + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            }
        }
        if constexpr (EPI == DM_MLP_EPI_GELU_FWD) {
#pragma unroll
            for (int j = 0; j < 64; ++j) v[j] = gelu(v[j]);
        }
        if constexpr (EPI == DM_MLP_EPI_GELU_BWD) {
            const float *pre = g.pre + z * g.pre_ms + row * g.ld_pre + n0;
#pragma unroll
            for (int j = 0; j < 64; j += 4) {
                const float4 u = *reinterpret_cast<const float4 *>(pre + j);
                v[j] *= gelu_grad(u.x);
                v[j + 1] *= gelu_grad(u.y);
                v[j + 2] *= gelu_grad(u.z);
                v[j + 3] *= gelu_grad(u.w);
            }
        }
        if constexpr (EPI == DM_MLP_EPI_GELU_FWD || EPI == DM_MLP_EPI_GELU_BWD) {
            if (g.out_bf16) {
                uint16_t *o = g.out_bf16 + z * g.bf16_ms + row * g.ld_bf16 + n0;
#pragma unroll
                for (int j = 0; j < 64; j += 8)
                    *reinterpret_cast<uint4 *>(o + j) = make_uint4(pack2(v[j], v[j + 1]), pack2(v[j + 2], v[j + 3]),
                                                                   pack2(v[j + 4], v[j + 5]), pack2(v[j + 6], v[j + 7]));
            }
            if (g.out_t) {   // column j of the tile: a warp writes 32 consecutive rows
                uint16_t *o = g.out_t + z * g.t_ms + int64_t(n0) * g.ld_t + row;
#pragma unroll
                for (int j = 0; j < 64; ++j) o[int64_t(j) * g.ld_t] = to_bf16(v[j]);
            }
        }
    } else if (pending) {
        // drain: wait (bounded) for the committed MMAs before the accumulator is released
        tcg::mbar_wait(tcg::smem_u32(&mbar), phase);
    }
    tcg::cp_async_wait_all();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kTmemCols));
}

// ---------------------------------------------------------------------------
// softmax, KL loss and its gradient: one CTA of 256 threads per row
// ---------------------------------------------------------------------------

constexpr int kRowThreads = 256;

__device__ __forceinline__ float block_reduce(float x, float *red, bool is_max) {
    for (int o = 16; o > 0; o >>= 1) {
        const float y = __shfl_xor_sync(0xffffffffu, x, o);
        x = is_max ? fmaxf(x, y) : x + y;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = x;
    __syncthreads();
    float r = red[0];
    for (int i = 1; i < kRowThreads / 32; ++i) r = is_max ? fmaxf(r, red[i]) : r + red[i];
    return r;
}

__global__ void __launch_bounds__(kRowThreads) softmax_kernel(const float *__restrict__ logits,
                                                              const float *__restrict__ targets, int rows, int nout,
                                                              float grad_scale, float *__restrict__ probs,
                                                              uint16_t *__restrict__ dz, uint16_t *__restrict__ dzt,
                                                              float *__restrict__ loss_rows) {
    __shared__ float red[kRowThreads / 32];
    const int64_t r = blockIdx.x, z = blockIdx.y;
    const int64_t base = (z * rows + r) * nout;
    constexpr int kMaxPer = 16;   // nout <= 16 * 256
    const int per = nout / kRowThreads;
    float x[kMaxPer];
    float mx = -INFINITY;
#pragma unroll
    for (int i = 0; i < kMaxPer; ++i)
        if (i < per) {
            x[i] = logits[base + threadIdx.x + i * kRowThreads];
            mx = fmaxf(mx, x[i]);
        }
    mx = block_reduce(mx, red, true);
    float sum = 0.f;
#pragma unroll
    for (int i = 0; i < kMaxPer; ++i)
        if (i < per) sum += expf(x[i] - mx);
    sum = block_reduce(sum, red, false);
    const float lse = logf(sum);
    float loss = 0.f;
#pragma unroll
    for (int i = 0; i < kMaxPer; ++i)
        if (i < per) {
            const int j = threadIdx.x + i * kRowThreads;
            const float lq = x[i] - mx - lse;
            const float q = expf(lq);
            if (probs) probs[base + j] = q;
            if (targets) {
                const float t = targets[base + j];
                if (t > 0.f) loss += t * (logf(t) - lq);
                const uint16_t d = to_bf16((q - t) * grad_scale);
                dz[base + j] = d;
                dzt[(z * nout + j) * rows + r] = d;
            }
        }
    if (targets && loss_rows) {
        loss = block_reduce(loss, red, false);
        if (threadIdx.x == 0) loss_rows[z * rows + r] = loss;
    }
}

// db[n] = sum_b d_t[n][b]: one warp per (n, member)
__global__ void bias_grad_kernel(const uint16_t *__restrict__ dt, int64_t ld, int64_t d_ms, int N, int rows,
                                 float *__restrict__ db, int64_t db_ms) {
    const int lane = threadIdx.x & 31;
    const int n = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t z = blockIdx.y;
    if (n >= N) return;
    const uint16_t *src = dt + z * d_ms + int64_t(n) * ld;
    float s = 0.f;
    for (int b = lane; b < rows; b += 32) s += from_bf16(src[b]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) db[z * db_ms + n] = s;
}

struct Layers {
    int n;
    int64_t w_off[8], b_off[8];
    int out[8], in[8];
};

__global__ void adam_kernel(float *__restrict__ params, const float *__restrict__ grads, float *__restrict__ m,
                            float *__restrict__ v, int64_t P, int64_t total, Layers L, float lr, float b1, float b2,
                            float eps, float c1, float c2, int step, uint16_t *__restrict__ wb,
                            uint16_t *__restrict__ wtb) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
        float p = params[i];
        if (step > 0) {
            const float gr = grads[i];
            const float mm = b1 * m[i] + (1.f - b1) * gr;
            const float vv = b2 * v[i] + (1.f - b2) * gr * gr;
            m[i] = mm;
            v[i] = vv;
            p -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
            params[i] = p;
        }
        const int64_t z = i / P, o = i - z * P;
        for (int l = 0; l < L.n; ++l) {
            const int64_t w = o - L.w_off[l];
            if (w >= 0 && w < int64_t(L.out[l]) * L.in[l]) {
                const int64_t rr = w / L.in[l], cc = w - rr * L.in[l];
                const uint16_t b = to_bf16(p);
                wb[i] = b;
                wtb[z * P + L.w_off[l] + cc * L.out[l] + rr] = b;
                break;
            }
        }
    }
}

__global__ void gather_kernel(const float *__restrict__ features, int nfeat, const float *__restrict__ targets,
                              int nout, int64_t samples, const int32_t *__restrict__ index, int rows, int width,
                              uint16_t *__restrict__ x, uint16_t *__restrict__ xt, float *__restrict__ t) {
    const int64_t r = blockIdx.x, z = blockIdx.y;
    int64_t s = index[z * rows + r];
    if (s < 0 || s >= samples) s = 0;   // an index outside the data set reads sample 0
    if (targets) {
        const float4 *src = reinterpret_cast<const float4 *>(targets + s * nout);
        float4 *dst = reinterpret_cast<float4 *>(t + (z * rows + r) * nout);
        for (int j = threadIdx.x; j < nout / 4; j += blockDim.x) dst[j] = src[j];
    }
    for (int f = threadIdx.x; f < width; f += blockDim.x) {
        const uint16_t b = to_bf16(f < nfeat ? features[s * nfeat + f] : 0.f);
        x[(z * rows + r) * width + f] = b;
        xt[(z * width + f) * rows + r] = b;
    }
}

__global__ void __launch_bounds__(kRowThreads) ensemble_kernel(const float *__restrict__ probs, int rows,
                                                               int members, int nout, const float *__restrict__ ref,
                                                               float *__restrict__ mean, float *__restrict__ spread,
                                                               float *__restrict__ tv_ref) {
    __shared__ float red[kRowThreads / 32];
    const int64_t r = blockIdx.x;
    float dev[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float dref = 0.f;
    for (int j = threadIdx.x; j < nout; j += kRowThreads) {
        float q[8];
        float mu = 0.f;
#pragma unroll
        for (int zz = 0; zz < 8; ++zz)
            if (zz < members) {
                q[zz] = probs[(int64_t(zz) * rows + r) * nout + j];
                mu += q[zz];
            }
        mu /= float(members);
        mean[r * nout + j] = mu;
#pragma unroll
        for (int zz = 0; zz < 8; ++zz)
            if (zz < members) dev[zz] += fabsf(q[zz] - mu);
        if (ref) dref += fabsf(mu - ref[r * nout + j]);
    }
    float sp = 0.f;
#pragma unroll
    for (int zz = 0; zz < 8; ++zz)
        if (zz < members) sp += block_reduce(dev[zz], red, false);
    if (threadIdx.x == 0) spread[r] = 0.5f * sp / float(members);
    if (ref) {
        dref = block_reduce(dref, red, false);
        if (threadIdx.x == 0) tv_ref[r] = 0.5f * dref;
    }
}

template <int EPI>
static int launch_gemm(const dm_mlp_gemm &g, int *status, cudaStream_t s) {
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(gemm_kernel<EPI>), int(kSmemBytes)) != cudaSuccess)
        return DM_ERR_CUDA;
    dim3 grid(g.M / kBM, g.N / kBN, g.members);
    gemm_kernel<EPI><<<grid, kThreads, kSmemBytes, s>>>(g, status);
    count_launch();
    return launch_status();
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }
static bool mult8(int64_t x) { return x >= 0 && (x & 7) == 0; }

}  // namespace mlp
}  // namespace dmg

using namespace dmg;

extern "C" int dm_mlp_gemm_run(const dm_mlp_gemm *g, int *status_dev, void *stream) {
    using namespace mlp;
    DM_CHECK_ARG(g && status_dev);
    DM_CHECK_ARG(g->M > 0 && g->N > 0 && g->K > 0 && g->members >= 1 && g->members <= 65535);
    DM_CHECK_ARG(g->M % kBM == 0 && g->N % kBN == 0 && g->K % kBK == 0 && g->M / kBM <= 65535);
    DM_CHECK_ARG(g->A && g->B && aligned16(g->A) && aligned16(g->B));
    DM_CHECK_ARG(mult8(g->lda) && mult8(g->ldb) && g->lda >= g->K && g->ldb >= g->K && mult8(g->a_ms) &&
                 mult8(g->b_ms));
    const bool bias = g->epi == DM_MLP_EPI_GELU_FWD || g->epi == DM_MLP_EPI_BIAS_F32;
    if (bias) DM_CHECK_ARG(g->bias != nullptr && g->bias_ms >= 0);
    if (g->out_f32) DM_CHECK_ARG(aligned16(g->out_f32) && g->ld_f32 >= g->N && (g->ld_f32 & 3) == 0 && (g->f32_ms & 3) == 0);
    if (g->out_bf16) DM_CHECK_ARG(aligned16(g->out_bf16) && g->ld_bf16 >= g->N && mult8(g->ld_bf16) && mult8(g->bf16_ms));
    if (g->out_t) DM_CHECK_ARG(g->ld_t >= g->M && g->t_ms >= 0);
    cudaStream_t s = as_stream(stream);
    switch (g->epi) {
        case DM_MLP_EPI_GELU_FWD:
            DM_CHECK_ARG(g->out_bf16 || g->out_t);
            return launch_gemm<DM_MLP_EPI_GELU_FWD>(*g, status_dev, s);
        case DM_MLP_EPI_BIAS_F32:
            DM_CHECK_ARG(g->out_f32);
            return launch_gemm<DM_MLP_EPI_BIAS_F32>(*g, status_dev, s);
        case DM_MLP_EPI_GELU_BWD:
            DM_CHECK_ARG(g->pre && aligned16(g->pre) && g->ld_pre >= g->N && (g->ld_pre & 3) == 0 &&
                         (g->pre_ms & 3) == 0 && (g->out_bf16 || g->out_t));
            return launch_gemm<DM_MLP_EPI_GELU_BWD>(*g, status_dev, s);
        case DM_MLP_EPI_F32:
            DM_CHECK_ARG(g->out_f32);
            return launch_gemm<DM_MLP_EPI_F32>(*g, status_dev, s);
        default:
            return DM_ERR_ARG;
    }
}

extern "C" int dm_mlp_softmax_xent(const float *logits, const float *targets, int rows, int members, int nout,
                                   float grad_scale, float *probs, uint16_t *dz, uint16_t *dzt, float *loss_rows,
                                   void *stream) {
    using namespace mlp;
    DM_CHECK_ARG(logits && rows > 0 && members >= 1 && members <= 65535 && nout > 0);
    DM_CHECK_ARG(nout % kRowThreads == 0 && nout <= 16 * kRowThreads);
    DM_CHECK_ARG(targets ? (dz && dzt) : (probs != nullptr));
    softmax_kernel<<<dim3(rows, members), kRowThreads, 0, as_stream(stream)>>>(logits, targets, rows, nout, grad_scale,
                                                                              probs, dz, dzt, loss_rows);
    count_launch();
    return launch_status();
}

extern "C" int dm_mlp_bias_grad(const uint16_t *d_t, int64_t ld, int64_t d_ms, int N, int rows, int members,
                                float *db, int64_t db_ms, void *stream) {
    DM_CHECK_ARG(d_t && db && N > 0 && rows > 0 && ld >= rows && members >= 1 && members <= 65535);
    const int warps = 8;
    mlp::bias_grad_kernel<<<dim3((N + warps - 1) / warps, members), 32 * warps, 0, as_stream(stream)>>>(
        d_t, ld, d_ms, N, rows, db, db_ms);
    count_launch();
    return launch_status();
}

extern "C" int dm_mlp_adam(float *params, const float *grads, float *m, float *v, int64_t count_per_member,
                           int members, const int32_t *shapes, int nlayers, float lr, float beta1, float beta2,
                           float eps, int step, uint16_t *w_bf16, uint16_t *wt_bf16, void *stream) {
    DM_CHECK_ARG(params && shapes && w_bf16 && wt_bf16 && members >= 1 && nlayers >= 1 && nlayers <= 8);
    DM_CHECK_ARG(step <= 0 || (grads && m && v));
    mlp::Layers L;
    L.n = nlayers;
    int64_t off = 0;
    for (int l = 0; l < nlayers; ++l) {
        DM_CHECK_ARG(shapes[2 * l] > 0 && shapes[2 * l + 1] > 0);
        L.out[l] = shapes[2 * l];
        L.in[l] = shapes[2 * l + 1];
        L.w_off[l] = off;
        off += int64_t(L.out[l]) * L.in[l];
        L.b_off[l] = off;
        off += L.out[l];
    }
    DM_CHECK_ARG(off == count_per_member);
    const double c1 = step > 0 ? 1.0 - pow(double(beta1), step) : 1.0;
    const double c2 = step > 0 ? 1.0 - pow(double(beta2), step) : 1.0;
    const int64_t total = count_per_member * members;
    mlp::adam_kernel<<<grid_for(total, 256), 256, 0, as_stream(stream)>>>(
        params, grads, m, v, count_per_member, total, L, lr, beta1, beta2, eps, float(c1), float(c2), step, w_bf16,
        wt_bf16);
    count_launch();
    return launch_status();
}

extern "C" int dm_mlp_gather(const float *features, int nfeat, const float *targets, int nout, int64_t samples,
                             const int32_t *index, int rows, int members, int width, uint16_t *x, uint16_t *xt,
                             float *t, void *stream) {
    DM_CHECK_ARG(features && index && x && xt && nfeat > 0 && nfeat <= width && samples > 0);
    DM_CHECK_ARG(rows > 0 && members >= 1 && members <= 65535 && width % 8 == 0 && nout > 0 && nout % 4 == 0);
    DM_CHECK_ARG(!targets || (t && mlp::aligned16(targets) && mlp::aligned16(t)));
    mlp::gather_kernel<<<dim3(rows, members), 256, 0, as_stream(stream)>>>(features, nfeat, targets, nout, samples,
                                                                          index, rows, width, x, xt, t);
    count_launch();
    return launch_status();
}

extern "C" int dm_mlp_ensemble(const float *probs, int rows, int members, int nout, const float *ref, float *mean,
                               float *spread, float *tv_ref, void *stream) {
    DM_CHECK_ARG(probs && mean && spread && rows > 0 && members >= 1 && members <= 8 && nout > 0);
    DM_CHECK_ARG(!ref || tv_ref);
    mlp::ensemble_kernel<<<rows, mlp::kRowThreads, 0, as_stream(stream)>>>(probs, rows, members, nout, ref, mean,
                                                                          spread, tv_ref);
    count_launch();
    return launch_status();
}
