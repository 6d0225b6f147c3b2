// Tensor-core fused pass (FP32 state, 3-way FP16 split on tcgen05).
//
// A pass holds 7 resident qubit axes: every tile of 4**7 = 16,384
// coefficients is streamed into shared memory (cp.async, 16-byte chunks),
// then the pass's register rounds run as matrix products on the tensor
// cores.  A round names 3 of the tile's axes; the round's operations,
// composed in FP64 on the device (compose_pass_kernel before the pass, or
// per instance inside the batched sweeps), form one 64x64 real transfer matrix U acting
// on the 64 coefficients that differ only in those axes.  With the tile
// viewed as 256 groups x 64 (one row per group), the round is
//     D[g][j'] = sum_j X[g][j] * U[j'][j]           (M = 256, N = 64, K = 64)
// issued as two M = 128 tcgen05.mma.kind::f16 chains into TMEM.  FP32
// accuracy comes from a 3-way FP16 split: inside the pass the tile is held
// in units of 2**-n (x = 2**n a, |x| <= 1), x = h + 2**-11 l with
// h = fp16(x), l = fp16(2**11 (x - h)), and U = Uh + 2**-11 Ul likewise;
//     D = h (2**11 Uh)^T + [h Ul^T + l Uh^T] = 2**11 x U^T + O(2**-22 |x|)
// (the l Ul term is below FP32), the large term and the bracketed
// corrections in separate FP32 accumulators, and the epilogue adds them and
// scales by 2**-11.
// FP16 runs at twice the TF32 rate and halves the operand bytes.  The
// epilogue reads D from TMEM (tcgen05.ld, one group per thread) and writes
// the h / l split directly in the operand layout of the next round.  The
// last round either stores each thread's row straight to global memory (a
// "direct" last round: its rows 0-3 are tile bits 0-3, so lanes 0-15 write
// 16 contiguous coefficients) while the next tile's cp.async load, issued as
// soon as the round's MMAs have read the operands, lands in the freed
// operand region; or, when it acts on local axes 0 and 1, it writes the tile
// back in its natural FP32 layout for 128-bit stores.  Every wait on an
// mbarrier is bounded: a wait that gives up records an error in *status and
// the kernel drains and returns.
//
// Two CTAs of 256 threads share an SM, so one CTA's tile load, barriers
// and MMA waits overlap the other's work.  Shared memory per CTA (dynamic,
// 88 KB): AH / AL 32 KB each (round operand h / l, K-major core-matrix FP16
// layout, 256 rows x 64; together they also hold the natural FP32 tile that
// cp.async streams in and the last round writes out), B 24 KB (2**11 Uh and
// Ul stacked as one 128-row operand, then Uh).  The h operand is read once
// per round for both of its terms (N = 128 into two 64-column accumulators
// that the epilogue adds); warps 0-3 own the rows of M block 0 and warps 4-7
// those of M block 1, one row per thread (TMEM lane quadrant = warp % 4).
#include <cuda_fp16.h>

#include <mutex>

#include "dm_batch.cuh"
#include "dm_common.cuh"
#include "dm_rounds.cuh"
#include "dm_tc_tile.cuh"
#include "dm_tcgen05.cuh"

namespace dmg {

namespace tc {

constexpr int kThreads = 256;                  // two CTAs per SM
constexpr int kCtasPerSm = 2;
constexpr int kBlocksPerThread = 256 / kThreads;   // M = 128 blocks in one thread's epilogue
constexpr uint32_t kBBytes = 3 * kBImage;      // 24 KB
constexpr uint32_t kSmemBytes = 2 * kABytes + kBBytes;   // 88 KB: two CTAs per SM
constexpr int kUHalves = 3 * 64 * 64;          // FP16 values per round image
constexpr uint32_t kTmemCols = 256;            // two M = 128 blocks x N = 128 (D1 | D2)

// Natural-layout swizzle of the tile (16-byte chunks intact), as in dm_pass.cu.
__device__ __forceinline__ int nat_swz(int e) { return e ^ ((((e >> 5) ^ (e >> 8)) & 7) << 2); }

struct Pass {
    int n, m, low, nrounds;
    int vec0;
    int direct;                      // the last round stores straight to global memory (offsets lastg)
    float up, down;                  // 2**n, 2**-n
    int64_t res_stride[kAxes];
    int64_t nonres_stride[DM_MAX_QUBITS];
    uint32_t natrow[8], natk[6];
    int64_t lastg[14];               // direct: global element offsets of the last round's row bits 0-7, K bits 0-5
    Round rounds[DM_MAX_ROUNDS];
};

// Global offsets of a direct last round's 14 bits: its tables hold the linear natural offset
// 2**b of tile bit b, i.e. bit b % 2 of local axis b / 2.
__host__ __device__ inline void direct_offsets(Pass &p, const uint32_t *rowc, const uint32_t *kc) {
    for (int i = 0; i < 14; ++i) {
        const uint32_t c = i < 8 ? rowc[i] : kc[i - 8];
        int b = 0;
        while (b < 2 * kAxes - 1 && (1u << b) != c) ++b;
        p.lastg[i] = p.res_stride[b >> 1] << (b & 1);
    }
}

__device__ __forceinline__ int64_t tile_offset(const Pass &p, int e) {
    int64_t off = e & ((1 << (2 * p.low)) - 1);
    for (int r = p.low; r < kAxes; ++r) off += int64_t((e >> (2 * r)) & 3) * p.res_stride[r];
    return off;
}

// Per-CTA tensor-core state shared by the single-state and the batched kernels.
struct TcCta {
    unsigned char *AH, *AL, *B;   // operand images h / l (the natural tile before and after the rounds), U
    uint64_t *mbar;               // MMA completion barrier
    int64_t *hi_off;              // kTile / 4 / kThreads chunk offsets of the current pass
    int *abort_s;                 // set when a bounded wait gave up
    uint32_t tmem;                // accumulator columns
    uint32_t phase;               // mbarrier phase to wait for next
    bool pending;                 // an MMA batch committed but not yet waited for
};

// mbarrier init and accumulator allocation (all threads).
__device__ __forceinline__ void tc_setup(TcCta &c, uint32_t *tmem_base_s) {
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        *c.abort_s = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(c.mbar)));
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_base_s)),
                     "n"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    c.tmem = *tmem_base_s;
    c.phase = 0;
    c.pending = false;
}

// Drain what is in flight and release the accumulator (all threads).
__device__ __forceinline__ void tc_teardown(TcCta &c) {
    if (c.pending) mbar_wait(smem_u32(c.mbar), c.phase);   // drain before the accumulator is released
    cp_async_wait_all();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "n"(kTmemCols));
}

// Streams tiles t0, t0 + dt, ... of one pass through the rounds (all threads
// of the CTA); round r's images are at umats + p.rounds[r].umoff.  Returns
// false when a bounded wait gave up (*status is then set).
__device__ __forceinline__ bool tc_pass_tiles(float *__restrict__ st, const Pass &p,
                                              const uint16_t *__restrict__ umats, int64_t t0, int64_t dt, TcCta &c,
                                              int *status) {
    unsigned char *AH = c.AH, *AL = c.AL, *B = c.B;
    uint64_t &mbar = *c.mbar;
    int64_t *hi_off = c.hi_off;
    volatile int &abort_s = *c.abort_s;
    const uint32_t tmem = c.tmem;
    uint32_t phase = c.phase;
    bool pending = c.pending;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int64_t ntiles = int64_t(1) << (2 * p.m);
    const int64_t off_tid = tile_offset(p, 4 * tid);
    __syncthreads();   // earlier readers of hi_off are done
    for (int i = tid; i < kTile / 4 / kThreads; i += kThreads) hi_off[i] = tile_offset(p, 4 * kThreads * i);
    __syncthreads();

    auto tile_base = [&](int64_t t) {
        int64_t base = 0;
        for (int u = 0; u < p.m; ++u) {
            base += (t & 3) * p.nonres_stride[u];
            t >>= 2;
        }
        return base;
    };
    auto load_tile = [&](int64_t t) {   // natural layout into AH / AL (64 KB)
        const float *src = st + tile_base(t) + off_tid;
#pragma unroll 8
        for (int i = 0; i < kTile / 4 / kThreads; ++i)
            cp_async16(AH + 4 * nat_swz(4 * (tid + kThreads * i)), src + hi_off[i]);
        cp_async_commit();
    };
    auto load_u = [&](int r) {          // round r's three U images into B (contiguous)
        const uint16_t *src = umats + p.rounds[r].umoff;
#pragma unroll
        for (int i = 0; i < int(kBBytes) / 16 / kThreads; ++i) {
            const int c = tid + kThreads * i;
            cp_async16(B + 16 * c, src + 8 * c);
        }
        cp_async_commit();
    };

    load_u(0);
    bool loaded = false;   // the tile's load went out during the previous tile's last round
    for (int64_t t = t0; t < ntiles; t += dt) {
        if (!loaded) load_tile(t);
        loaded = false;
        cp_async_wait_all();
        __syncthreads();
        // ---- natural tile -> round 0's operand (h / l), in place ----
        // Work items are (row, 8-value K chunk) pairs with the row's low three bits on the lane
        // bits, so each 16-byte chunk store of an 8-lane phase covers the 8 rows of one core
        // matrix: all 32 banks.  Every thread reads all of its values before any is written.
        {
            constexpr int kItems = kGroups * 8 / kThreads;   // 8
            const float *nat = reinterpret_cast<const float *>(AH);
            const float up = p.up;      // 2**n: the tile in units of 2**-n
            float x[kItems][8];
#pragma unroll
            for (int q = 0; q < kItems; ++q) {
                const int i = tid + kThreads * q;
                const int crow = ((i >> 6) << 3) | (i & 7), c = (i >> 3) & 7;
                // chunk c holds K = 8c .. 8c + 7: K bits 3-5 come from c, bits 0-2 from the element
                const uint32_t nb = xor_bits<8>(uint32_t(crow), p.natrow) ^ ((c & 1) ? p.natk[3] : 0u) ^
                                    ((c & 2) ? p.natk[4] : 0u) ^ ((c & 4) ? p.natk[5] : 0u);
                if (p.vec0 == 0) {   // digit 0 is local axis 0: four adjacent natural elements
                    const float4 a4 = *reinterpret_cast<const float4 *>(nat + nb);
                    const float4 b4 = *reinterpret_cast<const float4 *>(nat + (nb ^ p.natk[2]));
                    x[q][0] = a4.x; x[q][1] = a4.y; x[q][2] = a4.z; x[q][3] = a4.w;
                    x[q][4] = b4.x; x[q][5] = b4.y; x[q][6] = b4.z; x[q][7] = b4.w;
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        x[q][e] = nat[nb ^ ((e & 1) ? p.natk[0] : 0u) ^ ((e & 2) ? p.natk[1] : 0u) ^
                                      ((e & 4) ? p.natk[2] : 0u)];
                }
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < kItems; ++q) {
                const int i = tid + kThreads * q;
                const int crow = ((i >> 6) << 3) | (i & 7), c = (i >> 3) & 7;
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int e = 0; e < 8; e += 2) split2(x[q][e] * up, x[q][e + 1] * up, hw[e >> 1], lw[e >> 1]);
                const uint32_t o = row_off(crow) + uint32_t(c) * kLBO;
                *reinterpret_cast<uint4 *>(AH + o) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(AL + o) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        }
        for (int r = 0; r < p.nrounds; ++r) {
            // round 0's U was waited for with the tile; later rounds wait for their U
            if (r > 0) cp_async_wait_all();
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (tid == 0) {
                // D[:, 0:64] = h (2**11 Uh)^T and D[:, 64:128] = h Ul^T + l Uh^T: the h operand is
                // read once for both of its terms (N = 128 over the stacked images 2**11 Uh | Ul); the
                // large term's accumulator takes only its own four K steps, the two correction terms
                // (2**-11 smaller) share the other, and the epilogue adds the two in FP32
                const uint32_t ah = smem_u32(AH), al = smem_u32(AL), b0 = smem_u32(B);
#pragma unroll
                for (int mb = 0; mb < 2; ++mb) {
                    const uint32_t aoff = mb * (kABytes / 2);
#pragma unroll
                    for (int term = 0; term < 2; ++term) {
                        const uint32_t d = tmem + mb * 128 + (term == 0 ? 0u : 64u);
                        const uint32_t a = (term == 0 ? ah : al) + aoff;
                        const uint32_t b = b0 + term * 2 * kBImage;
                        const uint32_t idesc = term == 0 ? kIdesc128 : kIdesc64;
#pragma unroll
                        for (int ks = 0; ks < 4; ++ks) {      // K = 16 per MMA: two core matrices
                            const uint64_t da = smem_desc(a + ks * 2 * kLBO);
                            const uint64_t db = smem_desc(b + ks * 2 * kLBO);
                            const uint32_t acc = (term | ks) ? 1u : 0u;
                            asm volatile(
                                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                                "l"(da), "l"(db), "r"(idesc), "r"(acc));
                        }
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&mbar)));
            }
            pending = true;
            const bool ok = mbar_wait(smem_u32(&mbar), phase);
            if (ok) {
                phase ^= 1;
                pending = false;
            }
            if (!__all_sync(0xffffffffu, ok)) {
                if ((tid & 31) == 0) {
                    atomicExch(status, 1);
                    abort_s = 1;
                }
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            __syncthreads();
            if (abort_s) break;
            // B is free: fetch the next round's U (or round 0's, for the next tile)
            load_u(r + 1 < p.nrounds ? r + 1 : 0);
            // ---- epilogue: D -> next operand (h / l), or the natural tile after the last round ----
            // the thread holds row tid % 128 of M block tid / 128 (TMEM columns 0-127 / 128-255)
            const Round &R = p.rounds[r];
            uint32_t tk[3][4];
            digit_tables(R.kc, tk);
            const bool last = r + 1 == p.nrounds;
            if (last && p.direct && t + dt < ntiles) {
                // the operands are consumed and this round writes straight to global memory: the next
                // tile's load overlaps the epilogue
                load_tile(t + dt);
                loaded = true;
            }
#pragma unroll 1
            for (int i = 0; i < kBlocksPerThread; ++i) {
                const int mb = kBlocksPerThread == 1 ? (warp >> 2) : i;
                float v[64];
                const uint32_t ta = tmem + (uint32_t(32 * (warp & 3)) << 16) + uint32_t(mb * 128);
                // D[:, 0:64] + D[:, 64:128], 32 columns of each at a time (one wait per half)
                tcg::tmem_ld32_pair_add(ta, ta + 64, v);
                tcg::tmem_ld32_pair_add(ta + 32, ta + 96, v + 32);
                const uint32_t base = xor_bits<8>(uint32_t((tid & 127) + 128 * mb), R.rowc);
                if (!last) {
                    store_all<true>(v, R.vec, base, tk, AH, AL);   // split from the accumulator scale
                } else if (p.direct) {
                    // the row straight to global memory: rows 0-3 are tile bits 0-3 (16 contiguous
                    // coefficients on lanes 0-15)
                    const float down = p.down * kLoUnscale;
                    const int row = (tid & 127) + 128 * mb;
                    int64_t rowg = tile_base(t);
#pragma unroll
                    for (int b = 0; b < 8; ++b)
                        if ((row >> b) & 1) rowg += p.lastg[b];
                    float *row_ptr = st + rowg;
                    const int64_t k0 = p.lastg[8], k1 = p.lastg[9];
#pragma unroll
                    for (int d2 = 0; d2 < 4; ++d2) {
                        const int64_t o2 = (d2 & 1 ? p.lastg[12] : 0) + (d2 & 2 ? p.lastg[13] : 0);
#pragma unroll
                        for (int d1 = 0; d1 < 4; ++d1) {
                            float *q = row_ptr + o2 + (d1 & 1 ? p.lastg[10] : 0) + (d1 & 2 ? p.lastg[11] : 0);
                            const int j = 4 * d1 + 16 * d2;
                            q[0] = v[j] * down;
                            q[k0] = v[j + 1] * down;
                            q[k1] = v[j + 2] * down;
                            q[k0 + k1] = v[j + 3] * down;
                        }
                    }
                } else {
                    const float down = p.down * kLoUnscale;   // back to coefficients
#pragma unroll
                    for (int j = 0; j < 64; ++j) v[j] *= down;
                    store_all<false>(v, R.vec, base, tk, AH, AL);   // natural FP32 layout into AH / AL
                }
            }
            if (!last) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        }
        if (abort_s) break;
        if (p.direct) continue;   // written by the last round
        __syncthreads();
        // ---- write the tile back with 128-bit stores, each chunk's slot refilled with the next
        // tile's chunk as soon as it is read: a chunk is read and reloaded by the same thread ----
        {
            float *dst = st + tile_base(t) + off_tid;
            const float *out = reinterpret_cast<const float *>(AH);
            const bool next = t + dt < ntiles;
            const float *src = st + (next ? tile_base(t + dt) : 0) + off_tid;
#pragma unroll 8
            for (int i = 0; i < kTile / 4 / kThreads; ++i) {
                const int e = 4 * (tid + kThreads * i);
                const float4 v = *reinterpret_cast<const float4 *>(out + nat_swz(e));
                *reinterpret_cast<float4 *>(dst + hi_off[i]) = v;
                if (next) cp_async16(AH + 4 * nat_swz(e), src + hi_off[i]);
            }
            if (next) {
                cp_async_commit();
                loaded = true;
            }
        }
    }
    cp_async_wait_all();   // round 0's images prefetched for a tile that does not come
    __syncthreads();
    c.phase = phase;
    c.pending = pending;
    return !abort_s;
}

__global__ void __launch_bounds__(kThreads, kCtasPerSm)
    pass_tc_kernel(float *__restrict__ st, const __grid_constant__ Pass p, const uint16_t *__restrict__ umats,
                   int *status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int64_t hi_off[kTile / 4 / kThreads];
    __shared__ int abort_s;
    TcCta c{smem, smem + kABytes, smem + 2 * kABytes, &mbar, hi_off, &abort_s, 0, 0, false};
    tc_setup(c, &tmem_base_s);
    tc_pass_tiles(st, p, umats, blockIdx.x, gridDim.x, c, status);
    tc_teardown(c);
}

// ---------------------------------------------------------------------------
// batched sweeps on the tensor cores
// ---------------------------------------------------------------------------

constexpr int64_t kScratchHalves = int64_t(DM_MAX_ROUNDS) * kUHalves;   // round images per CTA

// Kernel parameters of one batched pass (thread 0 the scalars, all threads the rounds).
__device__ void batch_tc_setup(Pass &ps, const dm_batch_tc_pass &bp, int n) {
    const int tid = threadIdx.x;
    if (tid == 0) {
        ps.n = n;
        ps.m = n - kAxes;
        int low = 0;
        while (low < kAxes && bp.ops.axes[low] == n - 1 - low) ++low;
        ps.low = low;
        ps.nrounds = bp.ops.nrounds;
        ps.vec0 = bp.tables.vec0 == 0 ? 0 : -1;
        ps.direct = bp.tables.direct_last ? 1 : 0;
        ps.up = ldexpf(1.0f, n);
        ps.down = ldexpf(1.0f, -n);
        unsigned resident = 0;
        for (int r = 0; r < kAxes; ++r) {
            resident |= 1u << bp.ops.axes[r];
            ps.res_stride[r] = int64_t(1) << (2 * (n - 1 - bp.ops.axes[r]));
        }
        int m = 0;
        for (int q = n - 1; q >= 0; --q)
            if (!((resident >> q) & 1)) ps.nonres_stride[m++] = int64_t(1) << (2 * (n - 1 - q));
        for (int i = 0; i < 8; ++i) ps.natrow[i] = bp.tables.natrow[i];
        for (int i = 0; i < 6; ++i) ps.natk[i] = bp.tables.natk[i];
        if (ps.direct) {
            const dm_tc_round &L = bp.tables.rounds[bp.ops.nrounds - 1];
            direct_offsets(ps, L.rowc, L.kc);
        }
    }
    for (int r = tid; r < bp.ops.nrounds; r += kThreads) {
        const dm_tc_round &in = bp.tables.rounds[r];
        Round &o = ps.rounds[r];
        for (int i = 0; i < 3; ++i) o.digits[i] = in.digits[i];
        o.vec = in.vec;
        o.umoff = int32_t(r * kUHalves);
        for (int i = 0; i < 8; ++i) o.rowc[i] = in.rowc[i];
        for (int i = 0; i < 6; ++i) o.kc[i] = in.kc[i];
    }
}

// One operation on a 64-coefficient column in shared memory (index j = d0 +
// 4 d1 + 16 d2 over the round's digits; digit positions from the op flags),
// in FP64: the same maps as the register rounds, with runtime digits.
// Map2: 16x16 general maps too (the single-state passes; the batched plans hold none).
template <bool Map2>
__device__ void col_apply(double *col, const dm_op &op, const double *__restrict__ mats) {
    const double *mg = mats + op.moff;
    const int da = (op.flags >> 8) & 3, db = (op.flags >> 12) & 3;
    if (op.kind == DM_OP_MAP1) {
        double m[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) m[i] = mg[i];
        const int S = 1 << (2 * da);
#pragma unroll 1
        for (int o = 0; o < 16; ++o) {
            const int j0 = ((o >> (2 * da)) << (2 * da + 2)) | (o & (S - 1));
            double x0 = col[j0], x1 = col[j0 + S], x2 = col[j0 + 2 * S], x3 = col[j0 + 3 * S];
            map4(m, false, x0, x1, x2, x3);
            col[j0] = x0;
            col[j0 + S] = x1;
            col[j0 + 2 * S] = x2;
            col[j0 + 3 * S] = x3;
        }
        return;
    }
    const int SA = 1 << (2 * da), SB = 1 << (2 * db), SC = 1 << (2 * (3 - da - db));
    CxCoef<double> cx{1.0, 0.0, 1.0, 0.0, 0.0};
    const bool ideal = (op.flags & DM_CX_IDEAL) != 0;
    if (op.kind == DM_OP_CX && !ideal) cx = CxCoef<double>{mg[0], mg[1], mg[2], mg[3], mg[4]};
#pragma unroll 1
    for (int o = 0; o < 4; ++o) {   // the four groups of the third digit
        const int j0 = o * SC;
        double x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = col[j0 + (i >> 2) * SA + (i & 3) * SB];
        if (Map2 && op.kind == DM_OP_MAP2) {   // y[4 pa + pb] = sum_s mg[16 (4 pa + pb) + s] x[s]
#pragma unroll 1
            for (int i = 0; i < 16; ++i) {
                double acc = 0.0;
#pragma unroll
                for (int j = 0; j < 16; ++j) acc = fma(mg[16 * i + j], x[j], acc);
                col[j0 + (i >> 2) * SA + (i & 3) * SB] = acc;
            }
            continue;
        }
        if (op.kind == DM_OP_CX) {
            cx16(x, cx, ideal);
        } else {   // DM_OP_DIAG2: entry (pa, pb) scaled by mg[4 pa + pb]
#pragma unroll
            for (int i = 0; i < 16; ++i) x[i] *= mg[i];
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) col[j0 + (i >> 2) * SA + (i & 3) * SB] = x[i];
    }
}

// Round r's matrix U (64 x 64 in its K-digit order) is the round's operations
// applied to the 64 unit vectors: column k of U = ops(e_k), composed in FP64
// on a column held in shared memory, one thread per column.  Written as FP16
// images that the MMAs read, K-major (value (n%8)*8 + k%8 + (k/8)*64 +
// (n/8)*512 for output n, input k), with Uh = fp16(U) and
// Ul = fp16(2**11 (U - Uh)): three images 2**11 Uh | Ul | Uh for the
// cp.async-fed kernels, two images Uh | Ul for the TMA-fed one.
constexpr int kColStride = 65;   // doubles per column: a warp's 32 columns spread over the banks
static_assert(2 * 64 * kColStride * 8 <= int(kSmemBytes), "two rounds of FP64 columns fit the pass's shared memory");

template <bool Map2>
__device__ void compose_column(const dm_batch_pass &bp, int r, int k, const double *__restrict__ mats, double *col) {
#pragma unroll 1
    for (int j = 0; j < 64; ++j) col[j] = j == k ? 1.0 : 0.0;
    const int ob = r > 0 ? bp.round_end[r - 1] : 0, oe = bp.round_end[r];
    for (int o = ob; o < oe; ++o) col_apply<Map2>(col, bp.ops[o], mats);
}

__device__ void write_column(uint16_t *__restrict__ img, int k, const double *col, bool three) {
    const uint32_t kpos = uint32_t(k & 7) + uint32_t(k >> 3) * 64;
    const int uh = three ? 8192 : 0;   // three: 2**11 Uh at 0, Ul at 4096, Uh at 8192; two: Uh at 0, Ul at 4096
#pragma unroll 4
    for (int j = 0; j < 64; ++j) {
        const uint32_t pos = kpos + uint32_t(j & 7) * 8 + uint32_t(j >> 3) * 512;
        const double u = col[j];
        const __half h = __double2half(u);
        const double hd = double(__half2float(h));
        if (three) img[pos] = __half_as_ushort(__float2half_rn(float(hd * double(kLoScale))));
        img[4096 + pos] = __half_as_ushort(__double2half((u - hd) * double(kLoScale)));
        img[uh + pos] = __half_as_ushort(h);
    }
}

// All rounds of a batched pass into per-CTA scratch (three images per round),
// 128 threads, two rounds at a time; the pass's operand and matrix regions
// are free between passes.
__device__ void compose_rounds(const dm_batch_pass &bp, const double *__restrict__ mats, uint16_t *__restrict__ umats,
                               double *work) {
    const int nr = bp.nrounds;
    const int tid = threadIdx.x;
    if (tid >= 128) return;
    double *col = work + tid * kColStride;
    for (int r0 = 0; r0 < nr; r0 += 2) {
        const int r = r0 + (tid >> 6), k = tid & 63;
        if (r >= nr) break;
        compose_column<false>(bp, r, k, mats, col);
        write_column(umats + int64_t(r) * kUHalves, k, col, true);
    }
}

// One pass's round images for the single-state kernels: one CTA per round,
// one thread per column.
__global__ void __launch_bounds__(64)
    compose_pass_kernel(const __grid_constant__ dm_batch_pass bp, const double *__restrict__ mats,
                        uint16_t *__restrict__ images, int image_halves) {
    __shared__ double cols[64 * kColStride];
    const int r = blockIdx.x, k = threadIdx.x;
    double *col = cols + k * kColStride;
    compose_column<true>(bp, r, k, mats, col);
    write_column(images + int64_t(r) * image_halves, k, col, image_halves == kUHalves);
}

__global__ void __launch_bounds__(kThreads, kCtasPerSm)
    batch_tc_kernel(float *__restrict__ states, double *__restrict__ probs, const double *__restrict__ mats,
                    const dm_batch_instance *__restrict__ insts, int ninst, const dm_batch_tc_pass *__restrict__ passes,
                    int *counter, uint16_t *__restrict__ scratch, int *status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int64_t hi_off[kTile / 4 / kThreads];
    __shared__ int abort_s;
    __shared__ int inst_s;
    __shared__ Pass ps;
    TcCta c{smem, smem + kABytes, smem + 2 * kABytes, &mbar, hi_off, &abort_s, 0, 0, false};
    tc_setup(c, &tmem_base_s);
    uint16_t *umats = scratch + int64_t(blockIdx.x) * kScratchHalves;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) inst_s = atomicAdd(counter, 1);
        __syncthreads();
        const int ii = inst_s;
        if (ii >= ninst) break;
        const dm_batch_instance I = insts[ii];
        float *st = states + I.state_off;
        batch_init_zero<float, kThreads>(st, I.n);
        bool ok = true;
        for (int pi = 0; pi < I.npasses && ok; ++pi) {
            const dm_batch_tc_pass &bp = passes[I.pass_begin + pi];
            batch_tc_setup(ps, bp, I.n);
            compose_rounds(bp.ops, mats + I.mats_off, umats, reinterpret_cast<double *>(smem));
            __threadfence_block();
            __syncthreads();
            ok = tc_pass_tiles(st, ps, umats, 0, 1, c, status);
        }
        if (!ok) break;
        batch_z_readout<float, kThreads>(st, I.n, I.meas_err, probs + I.prob_off, reinterpret_cast<double *>(smem));
    }
    tc_teardown(c);
}

// Template sweeps on the tensor cores: per instance and pass, the slots'
// recipe chains are composed in FP64 (as in the CUDA-core template kernel)
// into shared memory, the round matrices composed from those coefficients,
// then the tiles streamed.  Slot s of the program is op s of the
// concatenated tensor-core passes; op o of a pass reads coef + 16 o.
constexpr int kCoefOffset = 2 * 64 * kColStride * 8;   // after the two rounds of FP64 columns
static_assert(kCoefOffset + DM_MAX_PASS_OPS * kCoefStride * 8 <= int(kSmemBytes), "slot coefficients fit");

__global__ void __launch_bounds__(kThreads, kCtasPerSm)
    batch_param_tc_kernel(float *__restrict__ states, double *__restrict__ probs, const dm_param_program P,
                          const dm_batch_tc_pass *__restrict__ passes, const double *__restrict__ params,
                          int params_stride, int ninst, int *counter, uint16_t *__restrict__ scratch, int *status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int64_t hi_off[kTile / 4 / kThreads];
    __shared__ int abort_s;
    __shared__ int inst_s;
    __shared__ Pass ps;
    __shared__ double prm[DM_PARAMS_MIN_STRIDE];
    TcCta c{smem, smem + kABytes, smem + 2 * kABytes, &mbar, hi_off, &abort_s, 0, 0, false};
    tc_setup(c, &tmem_base_s);
    uint16_t *umats = scratch + int64_t(blockIdx.x) * kScratchHalves;
    double *coef = reinterpret_cast<double *>(smem + kCoefOffset);
    const int tid = threadIdx.x;
    const int n = P.n;
    for (;;) {
        if (tid == 0) inst_s = atomicAdd(counter, 1);
        __syncthreads();
        const int ii = inst_s;
        if (ii >= ninst) break;
        if (tid < DM_PARAMS_MIN_STRIDE) prm[tid] = params[int64_t(ii) * params_stride + tid];
        float *st = states + (int64_t(ii) << (2 * n));
        batch_init_zero<float, kThreads>(st, n);   // its barriers also publish prm
        bool ok = true;
        int slot_base = 0;
        for (int pi = 0; pi < P.npasses && ok; ++pi) {
            const dm_batch_tc_pass &bp = passes[pi];
            batch_tc_setup(ps, bp, n);
            for (int o = tid; o < bp.ops.nops; o += kThreads)
                compose_slot(P, slot_base + o, prm, coef + o * kCoefStride);
            __syncthreads();
            compose_rounds(bp.ops, coef, umats, reinterpret_cast<double *>(smem));
            __threadfence_block();
            __syncthreads();
            ok = tc_pass_tiles(st, ps, umats, 0, 1, c, status);
            slot_base += bp.ops.nops;
        }
        if (!ok) break;
        batch_z_readout<float, kThreads>(st, n, prm[11], probs + (int64_t(ii) << n), reinterpret_cast<double *>(smem));
    }
    tc_teardown(c);
}

}  // namespace tc

}  // namespace dmg

using namespace dmg;

constexpr int kBatchTcMaxQubits = 12;   // the Z read-out's 2**n doubles fit the operand region

// Offsets must be distinct powers of two (operand) so that their XOR stays inside
// a 32 KB operand image, or natural-tile element offsets below 4**7.
static bool valid_tables(const uint32_t *rowc, const uint32_t *kc, int vec, bool natural) {
    uint32_t seen = 0;
    for (int i = 0; i < 14; ++i) {
        const uint32_t c = i < 8 ? rowc[i] : kc[i - 8];
        if (natural) {
            if (c == 0 || c >= uint32_t(tc::kTile)) return false;
        } else {
            if (c == 0 || (c & (c - 1)) || c >= tc::kABytes || (seen & c)) return false;
            seen |= c;
        }
    }
    if (vec >= 0) {
        if (vec > 2) return false;
        // natural: four FP32 elements (16 bytes); operand: four FP16 values (8 bytes)
        const uint32_t lo = natural ? 1 : 2, hi = natural ? 2 : 4, align = natural ? 4 : 8;
        if (kc[2 * vec] != lo || kc[2 * vec + 1] != hi) return false;
        for (int i = 0; i < 14; ++i) {   // the other bits keep 16-byte alignment
            if (i >= 8 && (i - 8) / 2 == vec) continue;
            const uint32_t c = i < 8 ? rowc[i] : kc[i - 8];
            if (c % align) return false;
        }
    }
    return true;
}

// A direct last round's tables: the linear natural offsets 2**b of 14 distinct tile bits, rows 0-3
// on tile bits 0-3 (lanes 0-15 of a warp store 16 contiguous coefficients).
static bool direct_tables(const uint32_t *rowc, const uint32_t *kc) {
    uint32_t seen = 0;
    for (int i = 0; i < 14; ++i) {
        const uint32_t c = i < 8 ? rowc[i] : kc[i - 8];
        if (c == 0 || (c & (c - 1)) || c >= uint32_t(tc::kTile) || (seen & c)) return false;
        seen |= c;
    }
    return (rowc[0] | rowc[1] | rowc[2] | rowc[3]) == 15u;
}

extern "C" int dm_apply_pass_tc(void *state_dev, int n, const dm_tc_pass *pass, const uint16_t *umats_dev,
                                size_t umats_count, int *status_dev, void *stream) {
    DM_CHECK_ARG(state_dev && pass && umats_dev && status_dev && valid_n(n));
    if (reinterpret_cast<uintptr_t>(state_dev) & 15 || reinterpret_cast<uintptr_t>(umats_dev) & 15) return DM_ERR_ARG;
    if (n < tc::kAxes) return DM_ERR_PROGRAM;
    const int nr = pass->nrounds;
    if (nr < 1 || nr > DM_MAX_ROUNDS) return DM_ERR_PROGRAM;
    static thread_local tc::Pass p;   // ~3.5 KB: keep it off the host stack
    bool resident[DM_MAX_QUBITS] = {false};
    for (int r = 0; r < tc::kAxes; ++r) {
        const int q = pass->axes[r];
        if (q < 0 || q >= n || (r > 0 && q >= pass->axes[r - 1])) return DM_ERR_PROGRAM;
        resident[q] = true;
        p.res_stride[r] = axis_stride(n, q);
    }
    int low = 0;
    while (low < tc::kAxes && pass->axes[low] == n - 1 - low) ++low;
    if (low < 1) return DM_ERR_PROGRAM;   // 16-byte chunks need the lowest axis resident
    p.low = low;
    p.n = n;
    p.m = n - tc::kAxes;
    p.up = float(ldexp(1.0, n));
    p.down = float(ldexp(1.0, -n));
    int m = 0;
    for (int q = n - 1; q >= 0; --q)
        if (!resident[q]) p.nonres_stride[m++] = axis_stride(n, q);
    for (int u = m; u < DM_MAX_QUBITS; ++u) p.nonres_stride[u] = 0;
    p.nrounds = nr;
    p.vec0 = pass->vec0 == 0 ? 0 : -1;
    p.direct = pass->direct_last ? 1 : 0;
    if (pass->direct_last != 0 && pass->direct_last != 1) return DM_ERR_PROGRAM;
    // round 0 conversion reads: natural offsets of round 0's bits
    if (!valid_tables(pass->natrow, pass->natk, p.vec0, true)) return DM_ERR_PROGRAM;
    for (int i = 0; i < 8; ++i) p.natrow[i] = pass->natrow[i];
    for (int i = 0; i < 6; ++i) p.natk[i] = pass->natk[i];
    for (int r = 0; r < nr; ++r) {
        const dm_tc_round &in = pass->rounds[r];
        tc::Round &o = p.rounds[r];
        for (int i = 0; i < 3; ++i) {
            if (in.digits[i] < 0 || in.digits[i] >= tc::kAxes) return DM_ERR_PROGRAM;
            o.digits[i] = in.digits[i];
        }
        o.vec = in.vec;
        const bool direct_round = p.direct && r + 1 == nr;
        if (!(direct_round ? direct_tables(in.rowc, in.kc) : valid_tables(in.rowc, in.kc, in.vec, r + 1 == nr)))
            return DM_ERR_PROGRAM;
        for (int i = 0; i < 8; ++i) o.rowc[i] = in.rowc[i];
        for (int i = 0; i < 6; ++i) o.kc[i] = in.kc[i];
        if (direct_round) tc::direct_offsets(p, in.rowc, in.kc);
        if (in.umoff < 0 || (in.umoff & 7) || size_t(in.umoff) + tc::kUHalves > umats_count) return DM_ERR_PROGRAM;
        o.umoff = in.umoff;
    }
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(tc::pass_tc_kernel), int(tc::kSmemBytes)) !=
        cudaSuccess)
        return DM_ERR_CUDA;
    const int64_t ntiles = int64_t(1) << (2 * p.m);
    // 88 KB of shared memory, <= 128 registers per thread and 256 TMEM columns per CTA: two CTAs per SM
    int64_t grid = int64_t(sm_count()) * tc::kCtasPerSm;
    if (grid > ntiles) grid = ntiles;
    tc::pass_tc_kernel<<<int(grid), tc::kThreads, tc::kSmemBytes, as_stream(stream)>>>(
        static_cast<float *>(state_dev), p, umats_dev, status_dev);
    count_launch();
    return launch_status();
}

extern "C" size_t dm_batch_tc_scratch_bytes(void) {
    return size_t(sm_count()) * tc::kCtasPerSm * size_t(tc::kScratchHalves) * sizeof(uint16_t);
}

// The rounds and operations of a tensor-core pass (round_axes[r][0..2] the
// round's local axes in K-digit order, each op on axes of its round, digit
// positions in its flags, coefficients inside mats_len values); 16x16
// general maps only where the caller composes them.
static int validate_round_ops(const dm_batch_pass &o, int64_t mats_len, bool map2) {
    if (o.nrounds < 1 || o.nrounds > DM_MAX_ROUNDS) return DM_ERR_PROGRAM;
    if (o.nops < 0 || o.nops > DM_MAX_PASS_OPS) return DM_ERR_PROGRAM;
    int prev_end = 0;
    for (int r = 0; r < o.nrounds; ++r) {
        for (int i = 0; i < 3; ++i) {
            const int a = o.round_axes[r][i];
            if (a < 0 || a >= tc::kAxes) return DM_ERR_PROGRAM;
            for (int j = 0; j < i; ++j)
                if (o.round_axes[r][j] == a) return DM_ERR_PROGRAM;
        }
        const int end = o.round_end[r];
        if (end < prev_end || end > o.nops) return DM_ERR_PROGRAM;
        for (int i = prev_end; i < end; ++i) {
            const dm_op &op = o.ops[i];
            int64_t need = 0;
            switch (op.kind) {
                case DM_OP_MAP1: need = 16; break;
                case DM_OP_DIAG2: need = 16; break;
                case DM_OP_CX: need = 5; break;
                case DM_OP_MAP2:
                    if (!map2) return DM_ERR_PROGRAM;
                    need = 256;
                    break;
                default: return DM_ERR_PROGRAM;
            }
            if (op.moff < 0 || op.moff + need > mats_len) return DM_ERR_PROGRAM;
            const int da = (op.flags >> 8) & 3, db = (op.flags >> 12) & 3;
            if (op.a < 0 || op.a >= tc::kAxes || da >= 3 || o.round_axes[r][da] != op.a) return DM_ERR_PROGRAM;
            if (op.kind != DM_OP_MAP1 &&
                (op.b < 0 || op.b >= tc::kAxes || op.b == op.a || db >= 3 || db == da || o.round_axes[r][db] != op.b))
                return DM_ERR_PROGRAM;
        }
        prev_end = end;
    }
    return prev_end == o.nops ? DM_OK : DM_ERR_PROGRAM;
}

// One tensor-core batched pass against an instance of n qubits with a coefficient block of mats_len values.
static int validate_batch_tc_pass(const dm_batch_tc_pass &bp, int n, int64_t mats_len) {
    const dm_batch_pass &o = bp.ops;
    if (o.k != tc::kAxes || o.nrounds < 1 || o.nrounds > DM_MAX_ROUNDS) return DM_ERR_PROGRAM;
    if (o.axes[0] != n - 1) return DM_ERR_PROGRAM;   // 16-byte chunks need the lowest axis resident
    for (int r = 0; r < tc::kAxes; ++r)
        if (o.axes[r] < 0 || o.axes[r] >= n || (r > 0 && o.axes[r] >= o.axes[r - 1])) return DM_ERR_PROGRAM;
    const int vec0 = bp.tables.vec0 == 0 ? 0 : -1;
    if (!valid_tables(bp.tables.natrow, bp.tables.natk, vec0, true)) return DM_ERR_PROGRAM;
    if (bp.tables.direct_last != 0 && bp.tables.direct_last != 1) return DM_ERR_PROGRAM;
    for (int r = 0; r < o.nrounds; ++r) {
        const dm_tc_round &tr = bp.tables.rounds[r];
        for (int i = 0; i < 3; ++i)
            if (tr.digits[i] != o.round_axes[r][i]) return DM_ERR_PROGRAM;
        const bool direct_round = bp.tables.direct_last && r + 1 == o.nrounds;
        if (!(direct_round ? direct_tables(tr.rowc, tr.kc) : valid_tables(tr.rowc, tr.kc, tr.vec, r + 1 == o.nrounds)))
            return DM_ERR_PROGRAM;
    }
    return validate_round_ops(o, mats_len, false);
}

extern "C" int dm_compose_rounds(int format, const dm_batch_pass *pass, const double *mats_dev, size_t mats_count,
                                 uint16_t *images_dev, size_t images_count, void *stream) {
    DM_CHECK_ARG(pass && mats_dev && images_dev && (format == DM_IMAGE_TC || format == DM_IMAGE_TMA));
    if (reinterpret_cast<uintptr_t>(images_dev) & 15 || reinterpret_cast<uintptr_t>(mats_dev) & 7) return DM_ERR_ARG;
    if (mats_count > size_t(INT32_MAX)) return DM_ERR_RANGE;
    const int rc = validate_round_ops(*pass, int64_t(mats_count), true);
    if (rc) return rc;
    const int halves = format == DM_IMAGE_TC ? tc::kUHalves : 2 * 4096;
    if (images_count < size_t(pass->nrounds) * size_t(halves)) return DM_ERR_ARG;
    tc::compose_pass_kernel<<<pass->nrounds, 64, 0, as_stream(stream)>>>(*pass, mats_dev, images_dev, halves);
    count_launch();
    return launch_status();
}

extern "C" int dm_batch_run_tc(float *states_dev, size_t states_count, double *probs_dev, size_t probs_count,
                               const double *mats_dev, size_t mats_count, const dm_batch_instance *insts_host,
                               const dm_batch_instance *insts_dev, int ninst, const dm_batch_tc_pass *passes_host,
                               const dm_batch_tc_pass *passes_dev, int npasses, int *counter_dev, void *scratch_dev,
                               size_t scratch_bytes, int *status_dev, void *stream) {
    DM_CHECK_ARG(states_dev && probs_dev && mats_dev && insts_host && insts_dev && passes_host && passes_dev &&
                 counter_dev && scratch_dev && status_dev && ninst >= 1 && npasses >= 1);
    if (reinterpret_cast<uintptr_t>(states_dev) & 15 || reinterpret_cast<uintptr_t>(scratch_dev) & 15) return DM_ERR_ARG;
    for (int i = 0; i < ninst; ++i) {
        const dm_batch_instance &I = insts_host[i];
        if (I.n < tc::kAxes || I.n > kBatchTcMaxQubits) return DM_ERR_RANGE;
        const int64_t total = int64_t(1) << (2 * I.n);
        if (I.state_off < 0 || (I.state_off & 3) || size_t(I.state_off + total) > states_count) return DM_ERR_ARG;
        if (I.prob_off < 0 || size_t(I.prob_off + (int64_t(1) << I.n)) > probs_count) return DM_ERR_ARG;
        if (I.mats_off < 0 || I.mats_len < 0 || size_t(I.mats_off + I.mats_len) > mats_count) return DM_ERR_ARG;
        if (I.npasses < 0 || I.pass_begin < 0 || I.pass_begin + I.npasses > npasses) return DM_ERR_PROGRAM;
        for (int p = 0; p < I.npasses; ++p) {
            const int rc = validate_batch_tc_pass(passes_host[I.pass_begin + p], I.n, I.mats_len);
            if (rc) return rc;
        }
    }
    if (scratch_bytes < dm_batch_tc_scratch_bytes()) return DM_ERR_ARG;
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(tc::batch_tc_kernel), int(tc::kSmemBytes)) !=
        cudaSuccess)
        return DM_ERR_CUDA;
    cudaStream_t s = as_stream(stream);
    DM_CUDA_TRY(cudaMemsetAsync(counter_dev, 0, sizeof(int), s));
    const int grid = sm_count() * tc::kCtasPerSm;
    tc::batch_tc_kernel<<<grid, tc::kThreads, tc::kSmemBytes, s>>>(states_dev, probs_dev, mats_dev, insts_dev, ninst,
                                                                     passes_dev, counter_dev,
                                                                     static_cast<uint16_t *>(scratch_dev), status_dev);
    count_launch();
    return launch_status();
}

extern "C" int dm_batch_run_params_tc(const dm_param_program *host, const dm_param_program *dev,
                                      const dm_batch_tc_pass *passes_host, const dm_batch_tc_pass *passes_dev,
                                      const double *params_dev, int params_stride, int ninst, float *states_dev,
                                      size_t states_count, double *probs_dev, size_t probs_count, int *counter_dev,
                                      void *scratch_dev, size_t scratch_bytes, int *status_dev, void *stream) {
    DM_CHECK_ARG(host && dev && passes_host && passes_dev && params_dev && states_dev && probs_dev && counter_dev &&
                 scratch_dev && status_dev);
    DM_CHECK_ARG(ninst >= 1 && params_stride >= DM_PARAMS_MIN_STRIDE);
    if (reinterpret_cast<uintptr_t>(states_dev) & 15 || reinterpret_cast<uintptr_t>(scratch_dev) & 15) return DM_ERR_ARG;
    const dm_param_program &P = *host;
    if (P.n < tc::kAxes || P.n > kBatchTcMaxQubits) return DM_ERR_RANGE;
    if (P.npasses < 1) return DM_ERR_PROGRAM;
    for (int p = 0; p < P.npasses; ++p) {
        // op o of a pass reads the o-th 16-value slot of the shared-memory coefficients
        const dm_batch_pass &o = passes_host[p].ops;
        if (o.nops < 0 || o.nops > DM_MAX_PASS_OPS) return DM_ERR_PROGRAM;
        for (int i = 0; i < o.nops; ++i)
            if (o.ops[i].moff != i * kCoefStride) return DM_ERR_PROGRAM;
        const int rc = validate_batch_tc_pass(passes_host[p], P.n, int64_t(o.nops) * kCoefStride);
        if (rc) return rc;
    }
    const int rc = validate_param_slots(
        P, P.npasses, [&](int p) { return int(passes_host[p].ops.nops); },
        [&](int p, int o) { return passes_host[p].ops.ops[o].kind; });
    if (rc) return rc;
    if (host->n != dev->n || host->npasses != dev->npasses || host->nslots != dev->nslots) return DM_ERR_ARG;
    if (size_t(ninst) * (size_t(1) << (2 * P.n)) > states_count) return DM_ERR_ARG;
    if (size_t(ninst) * (size_t(1) << P.n) > probs_count) return DM_ERR_ARG;
    if (scratch_bytes < dm_batch_tc_scratch_bytes()) return DM_ERR_ARG;
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(tc::batch_param_tc_kernel), int(tc::kSmemBytes)) !=
        cudaSuccess)
        return DM_ERR_CUDA;
    cudaStream_t s = as_stream(stream);
    DM_CUDA_TRY(cudaMemsetAsync(counter_dev, 0, sizeof(int), s));
    const int grid = sm_count() * tc::kCtasPerSm;
    tc::batch_param_tc_kernel<<<grid, tc::kThreads, tc::kSmemBytes, s>>>(
        states_dev, probs_dev, *dev, passes_dev, params_dev, params_stride, ninst, counter_dev,
        static_cast<uint16_t *>(scratch_dev), status_dev);
    count_launch();
    return launch_status();
}
