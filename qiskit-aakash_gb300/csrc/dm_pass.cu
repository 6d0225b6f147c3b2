// Gates and noise on the Pauli-coefficient vector.
//
// * map1_kernel / cx_kernel: one operation per sweep (the reference applies
//   every rotation, CX and noise channel as its own full-state numpy sweep,
//   basicaertools.py:93-126, :310-392; dm_simulator.py:397-425).
// * pass_kernel: the fused form.  The pass names k "resident" qubit axes; the
//   4**n vector splits into 4**(n-k) tiles of 4**k coefficients that differ
//   only in those axes.  One CTA loads a tile into shared memory, applies the
//   pass's whole operation list to it and writes it back: one HBM read and
//   one HBM write per coefficient for any number of operations on resident
//   axes.  Passes always include the lowest (contiguous) axes so that loads
//   and stores move whole 128-byte lines.
#include <mutex>

#include "dm_common.cuh"
#include "dm_batch.cuh"
#include "dm_rounds.cuh"

namespace dmg {

// ---------------------------------------------------------------------------
// operation bodies on a group of 4 or 16 coefficients
// ---------------------------------------------------------------------------

template <typename T>
struct Mat4 {
    T m[16];
};

// ---------------------------------------------------------------------------
// single-operation sweeps
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(256) map1_kernel(T *__restrict__ st, int log4s, int64_t ngroups,
                                                   Mat4<T> m, int row0_id) {
    const int64_t s = int64_t(1) << (2 * log4s);
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < ngroups;
         g += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i0 = ((g >> (2 * log4s)) << (2 * log4s + 2)) | (g & (s - 1));
        T x0 = st[i0], x1 = st[i0 + s], x2 = st[i0 + 2 * s], x3 = st[i0 + 3 * s];
        map4(m.m, row0_id != 0, x0, x1, x2, x3);
        st[i0] = x0;
        st[i0 + s] = x1;
        st[i0 + 2 * s] = x2;
        st[i0 + 3 * s] = x3;
    }
}

__device__ __forceinline__ int64_t insert_zero_digit(int64_t g, int pos) {
    const int64_t low = g & ((int64_t(1) << (2 * pos)) - 1);
    return ((g >> (2 * pos)) << (2 * pos + 2)) | low;
}

template <typename T>
__global__ void __launch_bounds__(256) cx_kernel(T *__restrict__ st, int pos_c, int pos_t, int64_t ngroups,
                                                 CxCoef<T> k, int ideal) {
    const int lo = pos_c < pos_t ? pos_c : pos_t;
    const int hi = pos_c < pos_t ? pos_t : pos_c;
    const int64_t sc = int64_t(1) << (2 * pos_c), stt = int64_t(1) << (2 * pos_t);
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < ngroups;
         g += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i0 = insert_zero_digit(insert_zero_digit(g, lo), hi);
        T x[16];
#pragma unroll
        for (int pc = 0; pc < 4; ++pc)
#pragma unroll
            for (int pt = 0; pt < 4; ++pt) x[4 * pc + pt] = st[i0 + pc * sc + pt * stt];
        cx16(x, k, ideal != 0);
#pragma unroll
        for (int pc = 0; pc < 4; ++pc)
#pragma unroll
            for (int pt = 0; pt < 4; ++pt) st[i0 + pc * sc + pt * stt] = x[4 * pc + pt];
    }
}

// ---------------------------------------------------------------------------
// fused pass
// ---------------------------------------------------------------------------

struct PassDev {
    int n, k, low, m, nops;
    int64_t res_stride[DM_MAX_TILE_AXES];      // global stride of local axis r
    int64_t nonres_stride[DM_MAX_QUBITS];      // global stride of tile-index digit u
    dm_op ops[DM_MAX_PASS_OPS];
};

__device__ __forceinline__ int64_t tile_offset(const PassDev &p, int e) {
    int64_t off = e & ((1 << (2 * p.low)) - 1);
    for (int r = p.low; r < p.k; ++r) off += int64_t((e >> (2 * r)) & 3) * p.res_stride[r];
    return off;
}

template <typename T>
__device__ void tile_map1(T *tile, int k, int r, const T *__restrict__ mg, bool row0_id) {
    T m[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = mg[i];
    const int s = 1 << (2 * r);
    const int ng = 1 << (2 * (k - 1));
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        const int i0 = ((g >> (2 * r)) << (2 * r + 2)) | (g & (s - 1));
        T x0 = tile[i0], x1 = tile[i0 + s], x2 = tile[i0 + 2 * s], x3 = tile[i0 + 3 * s];
        map4(m, row0_id, x0, x1, x2, x3);
        tile[i0] = x0;
        tile[i0 + s] = x1;
        tile[i0 + 2 * s] = x2;
        tile[i0 + 3 * s] = x3;
    }
}

__device__ __forceinline__ int insert_zero_digit32(int g, int pos) {
    return ((g >> (2 * pos)) << (2 * pos + 2)) | (g & ((1 << (2 * pos)) - 1));
}

template <typename T>
__device__ void tile_pair(T *tile, int k, const dm_op &op, const T *__restrict__ mg) {
    const int ra = op.a, rb = op.b;
    const int lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
    const int sa = 1 << (2 * ra), sb = 1 << (2 * rb);
    const int ng = 1 << (2 * (k - 2));
    CxCoef<T> cx;
    if (op.kind == DM_OP_CX) {
        cx.c = mg[0];
        cx.s = mg[1];
        cx.c2 = mg[2];
        cx.s2 = mg[3];
        cx.cs = mg[4];
    }
    const bool ideal = (op.flags & DM_CX_IDEAL) != 0;
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        const int i0 = insert_zero_digit32(insert_zero_digit32(g, lo), hi);
        T x[16];
#pragma unroll
        for (int pa = 0; pa < 4; ++pa)
#pragma unroll
            for (int pb = 0; pb < 4; ++pb) x[4 * pa + pb] = tile[i0 + pa * sa + pb * sb];
        if (op.kind == DM_OP_CX) {
            cx16(x, cx, ideal);
        } else {  // DM_OP_MAP2
            T y[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                T acc = T(0);
#pragma unroll
                for (int j = 0; j < 16; ++j) acc = fma(mg[16 * i + j], x[j], acc);
                y[i] = acc;
            }
#pragma unroll
            for (int i = 0; i < 16; ++i) x[i] = y[i];
        }
#pragma unroll
        for (int pa = 0; pa < 4; ++pa)
#pragma unroll
            for (int pb = 0; pb < 4; ++pb) tile[i0 + pa * sa + pb * sb] = x[4 * pa + pb];
    }
}

template <typename T>
__device__ void tile_diag2(T *tile, int k, int ra, int rb, const T *__restrict__ dg) {
    const int tsize = 1 << (2 * k);
    for (int e = threadIdx.x; e < tsize; e += blockDim.x) {
        const int pa = (e >> (2 * ra)) & 3, pb = (e >> (2 * rb)) & 3;
        tile[e] *= dg[4 * pa + pb];
    }
}

template <typename T>
__global__ void __launch_bounds__(256) pass_kernel(T *__restrict__ st, const __grid_constant__ PassDev p,
                                                   const T *__restrict__ mats) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *tile = reinterpret_cast<T *>(smem_raw);
    const int tsize = 1 << (2 * p.k);
    const int64_t ntiles = int64_t(1) << (2 * p.m);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int64_t base = 0;
        {
            int64_t tt = t;
            for (int u = 0; u < p.m; ++u) {
                base += (tt & 3) * p.nonres_stride[u];
                tt >>= 2;
            }
        }
        for (int e = threadIdx.x; e < tsize; e += blockDim.x) tile[e] = st[base + tile_offset(p, e)];
        __syncthreads();
        for (int i = 0; i < p.nops; ++i) {
            const dm_op &op = p.ops[i];
            const T *mg = mats + op.moff;
            if (op.kind == DM_OP_MAP1)
                tile_map1(tile, p.k, op.a, mg, (op.flags & DM_MAP1_ROW0_IDENTITY) != 0);
            else if (op.kind == DM_OP_DIAG2)
                tile_diag2(tile, p.k, op.a, op.b, mg);
            else
                tile_pair(tile, p.k, op, mg);
            __syncthreads();
        }
        for (int e = threadIdx.x; e < tsize; e += blockDim.x) st[base + tile_offset(p, e)] = tile[e];
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// fused pass with register rounds
//
// The pass's operations are grouped (on the host) into rounds; a round names
// R local axes (R = 3 for FP32: 64 coefficients, R = 2 for FP64: 16) and the
// consecutive operations that act only on them.  In a round every thread
// loads groups of 4**R coefficients spanning those axes from the shared tile
// into registers, applies all of the round's operations there and stores
// the group back: one shared-memory round trip per round instead of one per
// operation.
// ---------------------------------------------------------------------------

struct PassRounds {
    int n, k, low, m, nops, nrounds;
    int64_t res_stride[DM_MAX_TILE_AXES];
    int64_t nonres_stride[DM_MAX_QUBITS];
    int8_t rax[DM_MAX_ROUNDS][4];
    int16_t rend[DM_MAX_ROUNDS];
    dm_op ops[DM_MAX_PASS_OPS];
};

// Shared-memory position of tile element e: the low five bits are XORed
// with the next five, which spreads the groups of a warp over the 32 banks.
// swz is XOR-linear on elements with disjoint bits, so the position of
// (group base | round offset) is swz(base) ^ swz(offset).
__device__ __forceinline__ int swz(int e) { return e ^ ((e >> 5) & 31); }

__device__ __forceinline__ int64_t rounds_offset(const PassRounds &p, int e) {
    int64_t off = e & ((1 << (2 * p.low)) - 1);
    for (int r = p.low; r < p.k; ++r) off += int64_t((e >> (2 * r)) & 3) * p.res_stride[r];
    return off;
}

// Chunk-preserving swizzle: the 16-byte chunk index inside each 128-byte row
// is XORed with bits of the two next rows, so whole 16-byte chunks stay
// contiguous (cp.async / 128-bit accesses) while a warp's round groups
// spread over the banks.  XOR-linear on elements with disjoint bits.
template <typename T>
__device__ __forceinline__ int swz16(int e) {
    constexpr int C = sizeof(T) == 4 ? 2 : 1;   // log2(elements per 16-byte chunk)
    constexpr int S = C + 3;                      // first row bit (8 chunks per 128-byte row)
    return e ^ ((((e >> S) ^ (e >> (S + 3))) & 7) << C);
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int kPipeBuffers = 3;
constexpr int kPipeThreads = 256;

// Largest tile the pipelined kernel holds per buffer: 4**7 FP32 (64 KB) or 4**6 FP64 (32 KB).
template <typename T>
__host__ __device__ constexpr int pipe_tile_axes() { return sizeof(T) == 4 ? 7 : 6; }

// Stream tiles t0, t0 + dt, ... of one pass through kPipeBuffers shared
// buffers: while the rounds of tile i run, the 16-byte cp.async copies of
// the next tiles are in flight; each finished tile is written back with
// 128-bit stores.  Called by all threads of the CTA; bufs holds
// kPipeBuffers tiles of the dtype's largest pipelined tile, hi_off 64 int64.
template <typename T, int R>
__device__ __forceinline__ void pipe_tiles(T *__restrict__ st, const PassRounds &p, const T *__restrict__ mats,
                                           int64_t t0, int64_t dt, T *bufs, int64_t *hi_off) {
    constexpr int G = 1 << (2 * R);
    constexpr int CE = 16 / sizeof(T);                       // elements per 16-byte chunk
    constexpr int TMAX = 1 << (2 * pipe_tile_axes<T>());
    const int tsize = 1 << (2 * p.k);
    const int nchunks = tsize / CE;
    const int ngroups = 1 << (2 * (p.k - R));
    const int64_t ntiles = int64_t(1) << (2 * p.m);
    const int tid = threadIdx.x;
    // chunk c = tid + kPipeThreads * i covers elements e = CE * c ...: offset(e) = offset(CE*tid) + offset(CE*kPipeThreads*i)
    const int64_t off_tid = rounds_offset(p, (CE * tid) & (tsize - 1));
    __syncthreads();   // previous users of hi_off are done
    for (int i = tid; i < 64; i += kPipeThreads) {
        const int e = CE * kPipeThreads * i;
        hi_off[i] = e < tsize ? rounds_offset(p, e) : 0;
    }
    __syncthreads();

    auto tile_base = [&](int64_t t) {
        int64_t base = 0;
        for (int u = 0; u < p.m; ++u) {
            base += (t & 3) * p.nonres_stride[u];
            t >>= 2;
        }
        return base;
    };
    auto issue_load = [&](int64_t t, int b) {
        if (t < ntiles) {
            T *buf = bufs + b * TMAX;
            const T *src = st + tile_base(t) + off_tid;
            for (int i = 0; tid + kPipeThreads * i < nchunks; ++i) {
                const int e = CE * (tid + kPipeThreads * i);
                cp_async16(buf + swz16<T>(e), src + hi_off[i]);
            }
        }
        cp_async_commit();
    };

#pragma unroll
    for (int s = 0; s < kPipeBuffers - 1; ++s) issue_load(t0 + s * dt, s);
    int b = 0;
    for (int64_t t = t0; t < ntiles; t += dt) {
        cp_async_wait<kPipeBuffers - 2>();
        __syncthreads();
        // the buffer of the previous tile is free: start the copy that reuses it
        issue_load(t + (kPipeBuffers - 1) * dt, (b + kPipeBuffers - 1) % kPipeBuffers);
        T *tile = bufs + b * TMAX;
        int opb = 0;
        for (int r = 0; r < p.nrounds; ++r) {
            const int a0 = p.rax[r][0], a1 = p.rax[r][1], a2 = R > 2 ? p.rax[r][2] : 0;
            int t0s[4], t1s[4], t2s[4];
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                t0s[d] = swz16<T>(d << (2 * a0));
                t1s[d] = swz16<T>(d << (2 * a1));
                t2s[d] = R > 2 ? swz16<T>(d << (2 * a2)) : 0;
            }
            const int ope = p.rend[r];
            // With local axis 0 (the tile's fastest, 16-byte-chunk axis) as round digit 0, a
            // group's four values along it are one aligned 16-byte vector (FP32) or two (FP64).
            const bool vec = sizeof(T) == 4 && a0 == 0;
            for (int g = tid; g < ngroups; g += kPipeThreads) {
                int gb = insert_zero_digit32(g, a0);
                gb = insert_zero_digit32(gb, a1);
                if (R > 2) gb = insert_zero_digit32(gb, a2);
                int pb = swz16<T>(gb);
                T v[G];
                if (vec) {
#pragma unroll
                    for (int m = 0; m < G / 4; ++m) {
                        const float4 q = *reinterpret_cast<const float4 *>(tile + (pb ^ t1s[m & 3] ^ t2s[(m >> 2) & 3]));
                        v[4 * m] = q.x;
                        v[4 * m + 1] = q.y;
                        v[4 * m + 2] = q.z;
                        v[4 * m + 3] = q.w;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < G; ++j) v[j] = tile[pb ^ t0s[j & 3] ^ t1s[(j >> 2) & 3] ^ t2s[(j >> 4) & 3]];
                }
                for (int i = opb; i < ope; ++i) reg_apply<T, R>(v, p.ops[i], mats);
                asm volatile("" : "+r"(pb));   // recompute the addresses instead of keeping them live
                if (vec) {
#pragma unroll
                    for (int m = 0; m < G / 4; ++m)
                        *reinterpret_cast<float4 *>(tile + (pb ^ t1s[m & 3] ^ t2s[(m >> 2) & 3])) =
                            make_float4(v[4 * m], v[4 * m + 1], v[4 * m + 2], v[4 * m + 3]);
                } else {
#pragma unroll
                    for (int j = 0; j < G; ++j) tile[pb ^ t0s[j & 3] ^ t1s[(j >> 2) & 3] ^ t2s[(j >> 4) & 3]] = v[j];
                }
            }
            opb = ope;
            __syncthreads();
        }
        // write back with 128-bit stores (the next iteration's barrier orders
        // these reads before the buffer is refilled)
        T *dst = st + tile_base(t) + off_tid;
        for (int i = 0; tid + kPipeThreads * i < nchunks; ++i) {
            const int e = CE * (tid + kPipeThreads * i);
            *reinterpret_cast<float4 *>(dst + hi_off[i]) = *reinterpret_cast<const float4 *>(tile + swz16<T>(e));
        }
        b = (b + 1) % kPipeBuffers;
    }
    cp_async_wait<0>();
    __syncthreads();
}

// One persistent CTA per SM streams the pass's tiles.
template <typename T, int R>
__global__ void __launch_bounds__(kPipeThreads, 1) pass_pipe_kernel(T *__restrict__ st, const __grid_constant__ PassRounds p,
                                                                    const T *__restrict__ mats) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int64_t hi_off[64];
    pipe_tiles<T, R>(st, p, mats, blockIdx.x, gridDim.x, reinterpret_cast<T *>(smem_raw), hi_off);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static int build_pass(int n, const dm_pass *in, size_t mats_count, PassDev *out) {
    if (!in) return DM_ERR_ARG;
    const int k = in->k;
    if (k < 1 || k > DM_MAX_TILE_AXES || k > n) return DM_ERR_PROGRAM;
    if (in->nops < 0 || in->nops > DM_MAX_PASS_OPS) return DM_ERR_PROGRAM;
    bool resident[DM_MAX_QUBITS] = {false};
    for (int r = 0; r < k; ++r) {
        const int q = in->axes[r];
        if (q < 0 || q >= n) return DM_ERR_PROGRAM;
        if (r > 0 && q >= in->axes[r - 1]) return DM_ERR_PROGRAM;  // strictly decreasing
        resident[q] = true;
        out->res_stride[r] = axis_stride(n, q);
    }
    for (int r = k; r < DM_MAX_TILE_AXES; ++r) out->res_stride[r] = 0;
    int low = 0;
    while (low < k && in->axes[low] == n - 1 - low) ++low;
    int m = 0;
    for (int q = n - 1; q >= 0; --q)
        if (!resident[q]) out->nonres_stride[m++] = axis_stride(n, q);
    for (int u = m; u < DM_MAX_QUBITS; ++u) out->nonres_stride[u] = 0;
    for (int i = 0; i < in->nops; ++i) {
        const dm_op &op = in->ops[i];
        size_t need = 0;
        switch (op.kind) {
            case DM_OP_MAP1: need = 16; break;
            case DM_OP_MAP2: need = 256; break;
            case DM_OP_DIAG2: need = 16; break;
            case DM_OP_CX: need = 5; break;
            default: return DM_ERR_PROGRAM;
        }
        if (op.a < 0 || op.a >= k) return DM_ERR_PROGRAM;
        if (op.kind != DM_OP_MAP1 && (op.b < 0 || op.b >= k || op.b == op.a)) return DM_ERR_PROGRAM;
        if (op.moff < 0 || size_t(op.moff) + need > mats_count) return DM_ERR_PROGRAM;
        out->ops[i] = op;
    }
    out->n = n;
    out->k = k;
    out->low = low;
    out->m = n - k;
    out->nops = in->nops;
    return DM_OK;
}

// Validate the round structure of a pass and fill the kernel parameters.
static int build_rounds(const dm_pass *in, const PassDev &pd, int R, PassRounds *out) {
    const int nr = in->nrounds;
    if (nr < 1 || nr > DM_MAX_ROUNDS || pd.k < R) return DM_ERR_PROGRAM;
    // the pipelined kernel streams 16-byte chunks: the lowest qubit axis must be resident
    if (pd.low < 1 || pd.k > (R == DM_ROUND_AXES_F32 ? 7 : 6)) return DM_ERR_PROGRAM;
    int prev_end = 0;
    for (int r = 0; r < nr; ++r) {
        int last = -1;
        for (int i = 0; i < R; ++i) {
            const int a = in->round_axes[r][i];
            if (a <= last || a >= pd.k) return DM_ERR_PROGRAM;   // ascending, inside the tile
            last = a;
            out->rax[r][i] = int8_t(a);
        }
        for (int i = R; i < 4; ++i) out->rax[r][i] = -1;
        const int end = in->round_end[r];
        if (end < prev_end || end > pd.nops) return DM_ERR_PROGRAM;
        for (int o = prev_end; o < end; ++o) {
            const dm_op &op = in->ops[o];
            if (op.kind == DM_OP_MAP2) return DM_ERR_PROGRAM;   // not held in registers
            const int da = (op.flags >> 8) & 3, db = (op.flags >> 12) & 3;
            if (da >= R || in->round_axes[r][da] != op.a) return DM_ERR_PROGRAM;
            if (op.kind != DM_OP_MAP1 && (db >= R || db == da || in->round_axes[r][db] != op.b))
                return DM_ERR_PROGRAM;
        }
        out->rend[r] = int16_t(end);
        prev_end = end;
    }
    if (prev_end != pd.nops) return DM_ERR_PROGRAM;
    out->n = pd.n;
    out->k = pd.k;
    out->low = pd.low;
    out->m = pd.m;
    out->nops = pd.nops;
    out->nrounds = nr;
    for (int r = 0; r < DM_MAX_TILE_AXES; ++r) out->res_stride[r] = pd.res_stride[r];
    for (int u = 0; u < DM_MAX_QUBITS; ++u) out->nonres_stride[u] = pd.nonres_stride[u];
    for (int i = 0; i < pd.nops; ++i) out->ops[i] = pd.ops[i];
    return DM_OK;
}

template <typename T, int R>
static int launch_rounds(T *st, const PassRounds &p, const T *mats, cudaStream_t s) {
    const size_t smem = size_t(kPipeBuffers) * (size_t(1) << (2 * pipe_tile_axes<T>())) * sizeof(T);
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(pass_pipe_kernel<T, R>), int(smem)) != cudaSuccess)
        return DM_ERR_CUDA;
    const int64_t ntiles = int64_t(1) << (2 * p.m);
    int64_t grid = sm_count();
    if (grid > ntiles) grid = ntiles;
    pass_pipe_kernel<T, R><<<int(grid), kPipeThreads, smem, s>>>(st, p, mats);
    count_launch();
    return launch_status();
}

template <typename T>
static int launch_pass(T *st, const PassDev &p, const T *mats, cudaStream_t s) {
    const size_t smem = (size_t(1) << (2 * p.k)) * sizeof(T);
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(pass_kernel<T>),
                                int((size_t(1) << (2 * DM_MAX_TILE_AXES)) * sizeof(T))) != cudaSuccess)
        return DM_ERR_CUDA;
    int per_sm = 0;
    DM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pass_kernel<T>, 256, smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t ntiles = int64_t(1) << (2 * p.m);
    int64_t grid = int64_t(sm_count()) * per_sm;
    if (grid > ntiles) grid = ntiles;
    pass_kernel<T><<<int(grid), 256, smem, s>>>(st, p, mats);
    count_launch();
    return launch_status();
}

}  // namespace dmg

using namespace dmg;

extern "C" int dm_apply_pass(void *state_dev, int n, int dtype, const dm_pass *pass, const void *mats_dev,
                             size_t mats_count, void *stream) {
    DM_CHECK_ARG(state_dev && valid_n(n) && valid_dtype(dtype));
    DM_CHECK_ARG(mats_dev || mats_count == 0);
    PassDev p;
    int rc = build_pass(n, pass, mats_count, &p);
    if (rc) return rc;
    if (pass->nrounds > 0) {
        // the round kernel copies 16-byte chunks: the state must be 16-byte aligned
        if (reinterpret_cast<uintptr_t>(state_dev) & 15) return DM_ERR_ARG;
        static thread_local PassRounds pr;   // ~2.5 KB: keep it off the host stack
        const int R = dtype == DM_F64 ? DM_ROUND_AXES_F64 : DM_ROUND_AXES_F32;
        if ((rc = build_rounds(pass, p, R, &pr))) return rc;
        if (dtype == DM_F64)
            return launch_rounds<double, DM_ROUND_AXES_F64>(static_cast<double *>(state_dev), pr,
                                                            static_cast<const double *>(mats_dev), as_stream(stream));
        return launch_rounds<float, DM_ROUND_AXES_F32>(static_cast<float *>(state_dev), pr,
                                                       static_cast<const float *>(mats_dev), as_stream(stream));
    }
    if (dtype == DM_F64)
        return launch_pass(static_cast<double *>(state_dev), p, static_cast<const double *>(mats_dev),
                           as_stream(stream));
    return launch_pass(static_cast<float *>(state_dev), p, static_cast<const float *>(mats_dev),
                       as_stream(stream));
}

template <typename T>
static int do_map1(void *state_dev, int n, int q, const double *m4x4, cudaStream_t s) {
    Mat4<T> m;
    for (int i = 0; i < 16; ++i) m.m[i] = T(m4x4[i]);
    const bool row0_id = m4x4[0] == 1.0 && m4x4[1] == 0.0 && m4x4[2] == 0.0 && m4x4[3] == 0.0;
    const int64_t ngroups = pow4(n - 1);
    map1_kernel<T><<<grid_for(ngroups, 256), 256, 0, s>>>(static_cast<T *>(state_dev), n - 1 - q, ngroups, m,
                                                          row0_id ? 1 : 0);
    count_launch();
    return launch_status();
}

extern "C" int dm_apply_map1(void *state_dev, int n, int dtype, int q, const double *m4x4, void *stream) {
    DM_CHECK_ARG(state_dev && m4x4 && valid_n(n) && valid_dtype(dtype) && q >= 0 && q < n);
    return dtype == DM_F64 ? do_map1<double>(state_dev, n, q, m4x4, as_stream(stream))
                           : do_map1<float>(state_dev, n, q, m4x4, as_stream(stream));
}

// CX coefficients of the transition-selective-pulse model, basicaertools.py:329-336.
static void cx_coefficients(const double *err, double *c5, bool *ideal) {
    const double cav = err[0], mean = err[1];
    const double c2av = 4 * cav - 3;
    c5[0] = cav * cos(mean);
    c5[1] = cav * sin(mean);
    c5[2] = 0.5 * (1 + c2av * cos(2 * mean));
    c5[3] = 0.5 * (1 - c2av * cos(2 * mean));
    c5[4] = c2av * sin(mean) * cos(mean);
    *ideal = c5[0] == 1.0 && c5[1] == 0.0 && c5[2] == 1.0 && c5[3] == 0.0 && c5[4] == 0.0;
}

template <typename T>
static int do_cx(void *state_dev, int n, int qc, int qt, const double *err, cudaStream_t s) {
    double c5[5];
    bool ideal;
    cx_coefficients(err, c5, &ideal);
    CxCoef<T> k{T(c5[0]), T(c5[1]), T(c5[2]), T(c5[3]), T(c5[4])};
    const int64_t ngroups = pow4(n - 2);
    cx_kernel<T><<<grid_for(ngroups, 256), 256, 0, s>>>(static_cast<T *>(state_dev), n - 1 - qc, n - 1 - qt,
                                                        ngroups, k, ideal ? 1 : 0);
    count_launch();
    return launch_status();
}

extern "C" int dm_apply_cx(void *state_dev, int n, int dtype, int qc, int qt, const double *tsp_err2,
                           void *stream) {
    DM_CHECK_ARG(state_dev && tsp_err2 && valid_n(n) && valid_dtype(dtype));
    DM_CHECK_ARG(n >= 2 && qc >= 0 && qt >= 0 && qc < n && qt < n && qc != qt);
    return dtype == DM_F64 ? do_cx<double>(state_dev, n, qc, qt, tsp_err2, as_stream(stream))
                           : do_cx<float>(state_dev, n, qc, qt, tsp_err2, as_stream(stream));
}

extern "C" int dm_apply_memory_noise(void *state_dev, int n, int dtype, double f, double p, double g,
                                     void *stream) {
    DM_CHECK_ARG(state_dev && valid_n(n) && valid_dtype(dtype));
    const double k = sqrt(g) * f, d = (1 - g) * (2 * p - 1);
    const double m[16] = {1, 0, 0, 0, 0, k, 0, 0, 0, 0, k, 0, d, 0, 0, g};
    for (int q = 0; q < n; ++q) {
        int rc = dm_apply_map1(state_dev, n, dtype, q, m, stream);
        if (rc) return rc;
    }
    return DM_OK;
}

// ---------------------------------------------------------------------------
// batched sweeps: one persistent CTA per SM runs whole instances
// ---------------------------------------------------------------------------

namespace dmg {

constexpr int kBatchMaxQubits = 12;   // the Z read-out's 2**n doubles fit one tile buffer

// Kernel parameters of one batched pass (the resident axes' strides from the pass table).
template <int UNUSED = 0>
__device__ void batch_pass_setup(PassRounds &ps, const dm_batch_pass &bp, int n) {
    const int tid = threadIdx.x;
    if (tid == 0) {
        ps.n = n;
        ps.k = bp.k;
        ps.m = n - bp.k;
        ps.nops = bp.nops;
        ps.nrounds = bp.nrounds;
        int low = 0;
        while (low < bp.k && bp.axes[low] == n - 1 - low) ++low;
        ps.low = low;
        bool resident[DM_MAX_QUBITS] = {false};
        for (int r = 0; r < bp.k; ++r) {
            resident[bp.axes[r]] = true;
            ps.res_stride[r] = int64_t(1) << (2 * (n - 1 - bp.axes[r]));
        }
        int m = 0;
        for (int q = n - 1; q >= 0; --q)
            if (!resident[q]) ps.nonres_stride[m++] = int64_t(1) << (2 * (n - 1 - q));
    }
    for (int r = tid; r < bp.nrounds; r += kPipeThreads) {
        for (int i = 0; i < 4; ++i) ps.rax[r][i] = bp.round_axes[r][i];
        ps.rend[r] = bp.round_end[r];
    }
    for (int o = tid; o < bp.nops; o += kPipeThreads) ps.ops[o] = bp.ops[o];
}

template <typename T, int R>
__global__ void __launch_bounds__(kPipeThreads, 1)
    batch_kernel(T *__restrict__ states, double *__restrict__ probs, const T *__restrict__ mats,
                 const dm_batch_instance *__restrict__ insts, int ninst, const dm_batch_pass *__restrict__ passes,
                 int *counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int64_t hi_off[64];
    __shared__ PassRounds ps;
    __shared__ int inst_s;
    T *bufs = reinterpret_cast<T *>(smem_raw);
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) inst_s = atomicAdd(counter, 1);
        __syncthreads();
        const int ii = inst_s;
        if (ii >= ninst) break;
        const dm_batch_instance I = insts[ii];
        T *st = states + I.state_off;
        batch_init_zero<T, kPipeThreads>(st, I.n);
        for (int pi = 0; pi < I.npasses; ++pi) {
            batch_pass_setup(ps, passes[I.pass_begin + pi], I.n);
            __syncthreads();
            pipe_tiles<T, R>(st, ps, mats + I.mats_off, 0, 1, bufs, hi_off);
        }
        batch_z_readout<T, kPipeThreads>(st, I.n, I.meas_err, probs + I.prob_off, reinterpret_cast<double *>(smem_raw));
    }
}

// ---------------------------------------------------------------------------
// parametric programs: coefficients composed per instance and per pass
// ---------------------------------------------------------------------------

template <typename T, int R>
__global__ void __launch_bounds__(kPipeThreads, 1)
    batch_param_kernel(T *__restrict__ states, double *__restrict__ probs, const dm_param_program P,
                       const double *__restrict__ params, int params_stride, int ninst, int *counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int64_t hi_off[64];
    __shared__ PassRounds ps;
    __shared__ __align__(16) T coef[DM_MAX_PASS_OPS * kCoefStride];
    __shared__ double prm[DM_PARAMS_MIN_STRIDE];
    __shared__ int inst_s;
    T *bufs = reinterpret_cast<T *>(smem_raw);
    const int tid = threadIdx.x;
    const int n = P.n;
    for (;;) {
        if (tid == 0) inst_s = atomicAdd(counter, 1);
        __syncthreads();
        const int ii = inst_s;
        if (ii >= ninst) break;
        if (tid < DM_PARAMS_MIN_STRIDE) prm[tid] = params[int64_t(ii) * params_stride + tid];
        T *st = states + (int64_t(ii) << (2 * n));
        batch_init_zero<T, kPipeThreads>(st, n);     // its barriers also publish prm
        int slot_base = 0;
        for (int pi = 0; pi < P.npasses; ++pi) {
            const dm_batch_pass &bp = P.passes[pi];
            batch_pass_setup(ps, bp, n);
            for (int o = tid; o < bp.nops; o += kPipeThreads) {
                ps.ops[o].moff = o * kCoefStride;
                compose_slot(P, slot_base + o, prm, coef + o * kCoefStride);
            }
            __syncthreads();
            pipe_tiles<T, R>(st, ps, coef, 0, 1, bufs, hi_off);
            slot_base += bp.nops;
        }
        batch_z_readout<T, kPipeThreads>(st, n, prm[11], probs + (int64_t(ii) << n), reinterpret_cast<double *>(smem_raw));
    }
}

template <typename T, int R>
static int launch_batch(T *states, double *probs, const T *mats, const dm_batch_instance *insts, int ninst,
                        const dm_batch_pass *passes, int *counter, cudaStream_t s) {
    const size_t smem = size_t(kPipeBuffers) * (size_t(1) << (2 * pipe_tile_axes<T>())) * sizeof(T);
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(batch_kernel<T, R>), int(smem)) != cudaSuccess)
        return DM_ERR_CUDA;
    DM_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), s));
    int grid = sm_count();
    if (grid > ninst) grid = ninst;
    batch_kernel<T, R><<<grid, kPipeThreads, smem, s>>>(states, probs, mats, insts, ninst, passes, counter);
    count_launch();
    return launch_status();
}

// mats_len < 0: the pass's coefficients are composed on the device (moff is not read)
static int validate_batch_pass(const dm_batch_pass &bp, int n, int R, int kmax, int64_t mats_len) {
    const int k = bp.k;
    if (k < R || k > kmax || k > n) return DM_ERR_PROGRAM;
    if (bp.nops < 0 || bp.nops > DM_MAX_PASS_OPS || bp.nrounds < 1 || bp.nrounds > DM_MAX_ROUNDS) return DM_ERR_PROGRAM;
    if (bp.axes[0] != n - 1) return DM_ERR_PROGRAM;   // the lowest axis streams in 16-byte chunks
    for (int r = 0; r < k; ++r)
        if (bp.axes[r] < 0 || bp.axes[r] >= n || (r > 0 && bp.axes[r] >= bp.axes[r - 1])) return DM_ERR_PROGRAM;
    int prev_end = 0;
    for (int r = 0; r < bp.nrounds; ++r) {
        int last = -1;
        for (int i = 0; i < R; ++i) {
            const int a = bp.round_axes[r][i];
            if (a <= last || a >= k) return DM_ERR_PROGRAM;
            last = a;
        }
        const int end = bp.round_end[r];
        if (end < prev_end || end > bp.nops) return DM_ERR_PROGRAM;
        for (int o = prev_end; o < end; ++o) {
            const dm_op &op = bp.ops[o];
            int64_t need = 0;
            switch (op.kind) {
                case DM_OP_MAP1: need = 16; break;
                case DM_OP_DIAG2: need = 16; break;
                case DM_OP_CX: need = 5; break;
                default: return DM_ERR_PROGRAM;   // general 16x16 maps are not held in registers
            }
            if (mats_len >= 0 && (op.moff < 0 || op.moff + need > mats_len)) return DM_ERR_PROGRAM;
            const int da = (op.flags >> 8) & 3, db = (op.flags >> 12) & 3;
            if (op.a < 0 || op.a >= k || da >= R || bp.round_axes[r][da] != op.a) return DM_ERR_PROGRAM;
            if (op.kind != DM_OP_MAP1 &&
                (op.b < 0 || op.b >= k || op.b == op.a || db >= R || db == da || bp.round_axes[r][db] != op.b))
                return DM_ERR_PROGRAM;
        }
        prev_end = end;
    }
    return prev_end == bp.nops ? DM_OK : DM_ERR_PROGRAM;
}

template <typename T, int R>
static int launch_batch_params(T *states, double *probs, const dm_param_program &P, const double *params,
                               int params_stride, int ninst, int *counter, cudaStream_t s) {
    const size_t smem = size_t(kPipeBuffers) * (size_t(1) << (2 * pipe_tile_axes<T>())) * sizeof(T);
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(batch_param_kernel<T, R>), int(smem)) != cudaSuccess)
        return DM_ERR_CUDA;
    DM_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), s));
    int grid = sm_count();
    if (grid > ninst) grid = ninst;
    batch_param_kernel<T, R><<<grid, kPipeThreads, smem, s>>>(states, probs, P, params, params_stride, ninst, counter);
    count_launch();
    return launch_status();
}

// Every table of a parametric program: passes as for dm_batch_run, slots and
// recipe chains in range, and each slot's chain of a kind its op can take.
static int validate_param_program(const dm_param_program &P, int R, int kmax) {
    if (P.n < R || P.n > kBatchMaxQubits) return DM_ERR_RANGE;
    if (P.npasses < 0) return DM_ERR_PROGRAM;
    if (P.npasses && !P.passes) return DM_ERR_ARG;
    for (int p = 0; p < P.npasses; ++p) {
        const int rc = validate_batch_pass(P.passes[p], P.n, R, kmax, -1);
        if (rc) return rc;
    }
    return validate_param_slots(
        P, P.npasses, [&](int p) { return int(P.passes[p].nops); }, [&](int p, int o) { return P.passes[p].ops[o].kind; });
}

}  // namespace dmg

extern "C" int dm_batch_run(int dtype, void *states_dev, size_t states_count, double *probs_dev, size_t probs_count,
                            const void *mats_dev, size_t mats_count, const dm_batch_instance *insts_host,
                            const dm_batch_instance *insts_dev, int ninst, const dm_batch_pass *passes_host,
                            const dm_batch_pass *passes_dev, int npasses, int *counter_dev, int *status_dev,
                            void *stream) {
    DM_CHECK_ARG(valid_dtype(dtype) && states_dev && probs_dev && mats_dev && insts_host && insts_dev &&
                 passes_host && passes_dev && counter_dev && ninst >= 1 && npasses >= 1);
    (void)status_dev;
    if (reinterpret_cast<uintptr_t>(states_dev) & 15) return DM_ERR_ARG;
    const int R = dtype == DM_F64 ? DM_ROUND_AXES_F64 : DM_ROUND_AXES_F32;
    const int kmax = dtype == DM_F64 ? 6 : 7;
    for (int i = 0; i < ninst; ++i) {
        const dm_batch_instance &I = insts_host[i];
        if (I.n < R || I.n > kBatchMaxQubits) return DM_ERR_RANGE;
        const int64_t total = int64_t(1) << (2 * I.n);
        if (I.state_off < 0 || (I.state_off & 3) || size_t(I.state_off + total) > states_count) return DM_ERR_ARG;
        if (I.prob_off < 0 || size_t(I.prob_off + (int64_t(1) << I.n)) > probs_count) return DM_ERR_ARG;
        if (I.mats_off < 0 || I.mats_len < 0 || size_t(I.mats_off + I.mats_len) > mats_count) return DM_ERR_ARG;
        if (I.npasses < 0 || I.pass_begin < 0 || I.pass_begin + I.npasses > npasses) return DM_ERR_PROGRAM;
        for (int p = 0; p < I.npasses; ++p) {
            const int rc = validate_batch_pass(passes_host[I.pass_begin + p], I.n, R, kmax, I.mats_len);
            if (rc) return rc;
        }
    }
    cudaStream_t s = as_stream(stream);
    if (dtype == DM_F64)
        return launch_batch<double, DM_ROUND_AXES_F64>(static_cast<double *>(states_dev), probs_dev,
                                                       static_cast<const double *>(mats_dev), insts_dev, ninst,
                                                       passes_dev, counter_dev, s);
    return launch_batch<float, DM_ROUND_AXES_F32>(static_cast<float *>(states_dev), probs_dev,
                                                  static_cast<const float *>(mats_dev), insts_dev, ninst, passes_dev,
                                                  counter_dev, s);
}

extern "C" int dm_batch_run_params(int dtype, const dm_param_program *host, const dm_param_program *dev,
                                   const double *params_dev, int params_stride, int ninst, void *states_dev,
                                   size_t states_count, double *probs_dev, size_t probs_count, int *counter_dev,
                                   void *stream) {
    DM_CHECK_ARG(valid_dtype(dtype) && host && dev && params_dev && states_dev && probs_dev && counter_dev);
    DM_CHECK_ARG(ninst >= 1 && params_stride >= DM_PARAMS_MIN_STRIDE);
    if (reinterpret_cast<uintptr_t>(states_dev) & 15) return DM_ERR_ARG;
    const int R = dtype == DM_F64 ? DM_ROUND_AXES_F64 : DM_ROUND_AXES_F32;
    const int kmax = dtype == DM_F64 ? 6 : 7;
    const int rc = validate_param_program(*host, R, kmax);
    if (rc) return rc;
    if (host->n != dev->n || host->npasses != dev->npasses || host->nslots != dev->nslots) return DM_ERR_ARG;
    if (size_t(ninst) * (size_t(1) << (2 * host->n)) > states_count) return DM_ERR_ARG;
    if (size_t(ninst) * (size_t(1) << host->n) > probs_count) return DM_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    if (dtype == DM_F64)
        return launch_batch_params<double, DM_ROUND_AXES_F64>(static_cast<double *>(states_dev), probs_dev, *dev,
                                                              params_dev, params_stride, ninst, counter_dev, s);
    return launch_batch_params<float, DM_ROUND_AXES_F32>(static_cast<float *>(states_dev), probs_dev, *dev, params_dev,
                                                         params_stride, ninst, counter_dev, s);
}
