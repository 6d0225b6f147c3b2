// Tensor-core fused pass fed by TMA (FP32 state, 3-way FP16 split on tcgen05).
//
// Same arithmetic as pass_tc_kernel (dm_tc.cu): a pass holds 7 resident
// qubit axes; each tile of 4**7 = 16,384 coefficients runs the pass's rounds,
// each round a 64x64 real transfer matrix U on 3 of the tile's axes, issued
// as tcgen05.mma.kind::f16 over a 3-way FP16 split (tile in units of 2**-n,
// x = h + 2**-11 l; U = Uh + 2**-11 Ul):
//     D1 = h Uh^T,   D2 = h Ul^T + l Uh^T,   2**11 x U^T = 2**11 D1 + D2 + O(2**-22 |x|),
// D1 and D2 in separate FP32 accumulators (TMEM), combined by one FMA in the
// epilogue, which writes the next round's h / l operand (or, after the last
// round, the natural FP32 tile).
//
// What differs is how the work is fed and overlapped:
// * one persistent CTA per SM with two teams of 256 threads; each team owns
//   one 64 KB tile slot and 256 TMEM columns and streams its own tiles, so
//   one team's MMAs, loads and stores overlap the other team's epilogues;
// * tiles arrive by TMA (cp.async.bulk.tensor, completing on an mbarrier):
//   one thread of the team issues the load of its next tile as soon as the
//   last round's MMAs have read the slot, so the load overlaps the last
//   round's epilogue; that epilogue writes each thread's row straight to
//   global memory (lanes 0-15 on 16 contiguous coefficients);
// * the pass's round images ([Uh ; Ul], 16 KB per round) are loaded once per
//   CTA by bulk copies and stay in shared memory for the whole pass when it
//   has up to kUSlots rounds; a longer pass keeps its first kStreamFrom rounds
//   resident and streams each later round's image, per team, into one spare
//   slot (loaded as soon as the previous round's MMAs have read that slot).
// (An L2 prefetch of the next tile by cp.async.bulk.prefetch.tensor, tried in
// several forms, made the step slower: its issue holds the issuing thread,
// and with it the team, for thousands of cycles.)
//
// Tensor map.  The state is a 4**n vector whose flat index is the base-4
// number of the qubits' Pauli labels (qubit n-1 the lowest digit).  The 7
// resident digits form runs of consecutive positions; each run is split into
// chunks of at most 4 digits (a box dimension of <= 256 elements), and each
// chunk is one tensor-map dimension with stride 4**start elements, box
// 4**len and extent 4**(len + gap), where gap counts the non-resident digits
// directly above the chunk.  Tile t (its non-resident digits in increasing
// position order) has coordinate ((t >> 2 g) & (4**gap - 1)) * 4**len in that
// dimension, g being the number of non-resident digits below the gap.  The box
// lands in shared memory densely in dimension order, which is the tile's
// natural order (local axis r = the r-th lowest resident digit), unswizzled.
// The lowest digit is always resident, so every coordinate of dimension 0 is
// a multiple of 4 elements (16 bytes), as TMA requires.
//
// Shared memory (dynamic, 1024-byte aligned): slot 0 | slot 1 (64 KB each:
// AH | AL, 32 KB per FP16 operand image; the natural FP32 tile on load) |
// round images (16 KB per round).  Every mbarrier wait is bounded in time; a
// wait that gives up sets *status, the team stops, drains what it has in
// flight (MMA, tile load, round image) and the kernel returns.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>

#include "dm_common.cuh"
#include "dm_tc_tile.cuh"
#include "dm_tcgen05.cuh"

namespace dmg {

namespace tma {

using namespace tc;
using tcg::mbar_wait;
using tcg::smem_u32;

constexpr int kTeams = 2;
constexpr int kTeamThreads = 256;
constexpr int kThreads = kTeams * kTeamThreads;
constexpr int kMaxRounds = 16;                               // rounds of one pass
constexpr int kUSlots = 6;                                   // round-image slots in shared memory
constexpr int kStreamFrom = 4;                               // longer passes: rounds >= 4 streamed (slot 4 + team)
constexpr int kMaxDims = 5;                                  // tensor-map rank
constexpr uint32_t kSlotBytes = 2 * kABytes;                 // 64 KB: AH | AL, or the FP32 tile
constexpr uint32_t kUBytes = 2 * kBImage;                    // 16 KB per round: Uh | Ul (one 128-row operand)
constexpr uint32_t kUHalves = kUBytes / 2;
constexpr uint32_t kSmemBytes = kTeams * kSlotBytes + kUSlots * kUBytes + 1024;   // + alignment slack
constexpr uint32_t kTmemCols = 512;                          // per team: two M = 128 blocks x (D1 | D2)

struct TmaPass {
    int nrounds, ndims;
    int nres;                        // rounds whose images stay resident (all of them, or kStreamFrom)
    int last_vec;                    // the last round's K digit 0 is local axis 0: 16-byte stores
    float up, down;                  // 2**n, 2**-n
    int64_t ntiles;
    int8_t gap_first[kMaxDims];      // tile-index digit of the first non-resident digit above dimension i
    int8_t gap_len[kMaxDims];        // non-resident digits above dimension i
    int8_t box_log4[kMaxDims];       // resident digits of dimension i
    int8_t start[kMaxDims];          // digit position of dimension i (its stride is 4**start elements)
    int32_t uoff[kMaxRounds];        // FP16-value offset of round r's images
    uint32_t natrow[8], natk[6];     // round 0: natural-tile element offsets of its row and K bits
    int64_t lastg[14];               // last round: global element offsets of its row bits 0-7 and K bits 0-5
    Round rounds[kMaxRounds];
};

__device__ __forceinline__ void tile_coords(const TmaPass &p, int64_t t, int (&c)[kMaxDims]) {
#pragma unroll
    for (int i = 0; i < kMaxDims; ++i) {
        const int64_t g = (t >> (2 * p.gap_first[i])) & ((int64_t(1) << (2 * p.gap_len[i])) - 1);
        c[i] = int(g << (2 * p.box_log4[i]));
    }
}

// Global element offset of tile t's first coefficient (its non-resident digits).
__device__ __forceinline__ int64_t tile_base(const TmaPass &p, const int (&c)[kMaxDims]) {
    int64_t b = 0;
#pragma unroll
    for (int i = 0; i < kMaxDims; ++i) b += int64_t(c[i]) << (2 * p.start[i]);
    return b;
}

// TMA tile load of tile coordinates c into shared memory at dst, completing on mbar.
__device__ __forceinline__ void tma_load(const CUtensorMap *map, int nd, const int (&c)[kMaxDims], uint32_t dst,
                                         uint32_t mbar) {
    const uint64_t m = reinterpret_cast<uint64_t>(map);
    switch (nd) {
    case 1:
        asm volatile("cp.async.bulk.tensor.1d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];"
                     ::"r"(dst), "l"(m), "r"(c[0]), "r"(mbar) : "memory");
        break;
    case 2:
        asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                     "[%4];" ::"r"(dst), "l"(m), "r"(c[0]), "r"(c[1]), "r"(mbar) : "memory");
        break;
    case 3:
        asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                     "%4}], [%5];" ::"r"(dst), "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(mbar) : "memory");
        break;
    case 4:
        asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                     "%4, %5}], [%6];" ::"r"(dst), "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(mbar)
                     : "memory");
        break;
    default:
        asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
                     "%4, %5, %6}], [%7];" ::"r"(dst), "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]),
                     "r"(mbar) : "memory");
        break;
    }
}

__device__ __forceinline__ void team_sync(int team) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + team), "n"(kTeamThreads) : "memory");
}

// Barrier of the team that also ANDs `ok` over its threads: every thread of the
// team gets the same answer, so a failed wait anywhere sends the whole team
// down the same path (its barrier sequence stays matched).
__device__ __forceinline__ bool team_and(bool ok, int team) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.and.pred q, %2, %3, p;\nselp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"(uint32_t(ok)), "r"(1 + team), "n"(kTeamThreads)
        : "memory");
    return r != 0;
}

__global__ void __launch_bounds__(kThreads, 1)
    pass_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                    const __grid_constant__ TmaPass p,
                    float *__restrict__ st, const uint16_t *__restrict__ umats, int *status) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t load_bar[kTeams];
    __shared__ __align__(8) uint64_t mma_bar[kTeams];
    __shared__ __align__(8) uint64_t u_bar;
    __shared__ __align__(8) uint64_t stream_bar[kTeams];
    __shared__ uint32_t tmem_base_s;
    __shared__ volatile int pipe_busy;      // team 0's MMAs are in flight (a scheduling hint for team 1)
    unsigned char *smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int team = tid / kTeamThreads, ttid = tid % kTeamThreads;
    const bool leader = ttid == 0;
    unsigned char *AH = smem + team * kSlotBytes, *AL = AH + kABytes;
    unsigned char *U = smem + kTeams * kSlotBytes;
    const uint32_t lbar = smem_u32(&load_bar[team]), mbar = smem_u32(&mma_bar[team]), ubar = smem_u32(&u_bar);
    const uint32_t sbar = smem_u32(&stream_bar[team]);
    // round r's images: resident slot r, or this team's streaming slot
    auto uslot = [&](int r) -> uint32_t {
        return smem_u32(U + (r < p.nres ? r : kStreamFrom + team) * kUBytes);
    };

    if (tid == 0) {
        for (int i = 0; i < kTeams; ++i) {
            tcg::mbar_init(smem_u32(&load_bar[i]), 1);
            tcg::mbar_init(smem_u32(&mma_bar[i]), 1);
            tcg::mbar_init(smem_u32(&stream_bar[i]), 1);
        }
        tcg::mbar_init(ubar, 1);
        pipe_busy = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "n"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s + uint32_t(team * 256);

    const int64_t stride = int64_t(gridDim.x) * kTeams;
    int64_t t = int64_t(blockIdx.x) * kTeams + team;
    if (tid == 0) {   // the pass's round images, once per CTA
        tcg::mbar_expect_tx(ubar, uint32_t(p.nres) * kUBytes);
        for (int r = 0; r < p.nres; ++r)
            tcg::bulk_load(smem_u32(U + r * kUBytes), umats + p.uoff[r], kUBytes, ubar);
    }
    if (leader && t < p.ntiles) {
        int c[kMaxDims];
        tile_coords(p, t, c);
        tcg::mbar_expect_tx(lbar, kSlotBytes);
        tma_load(&tmap, p.ndims, c, smem_u32(AH), lbar);
    }
    bool load_pending = t < p.ntiles;
    bool mma_pending = false;
    bool u_pending = false;                 // a streamed round image in flight (leader)
    uint32_t lphase = 0, mphase = 0, uphase = 0;
    auto stream_u = [&](int r) {            // leader: round r's images into the team's streaming slot
        tcg::mbar_expect_tx(sbar, kUBytes);
        tcg::bulk_load(uslot(r), umats + p.uoff[r], kUBytes, sbar);
        u_pending = true;
    };
    const bool u_ok = team_and(mbar_wait(ubar, 0), team);
    if (!u_ok && ttid == 0) atomicExch(status, 1);

    // operand descriptors of the two M = 128 blocks of h and l (shared addresses < 256 KB: the
    // start-address field never carries into the next field)
    uint64_t adesc_h[2], adesc_l[2];
#pragma unroll
    for (int mb = 0; mb < 2; ++mb) {
        adesc_h[mb] = smem_desc(smem_u32(AH) + mb * (kABytes / 2));
        adesc_l[mb] = smem_desc(smem_u32(AL) + mb * (kABytes / 2));
    }

    // epilogue geometry: the thread holds row ttid of the 256-row operand, i.e. row ttid % 128 of
    // M block ttid / 128, in TMEM lane quadrant warp % 4
    const int mb_own = ttid >> 7;
    const uint32_t taddr = tmem + (uint32_t(32 * (warp & 3)) << 16) + uint32_t(mb_own * 128);

    for (; u_ok && t < p.ntiles; t += stride) {
        if (!team_and(mbar_wait(lbar, lphase), team)) {
            if (ttid == 0) atomicExch(status, 1);
            break;
        }
        lphase ^= 1;
        load_pending = false;
        const int64_t tn = t + stride;
        if (leader && p.nrounds > p.nres) stream_u(p.nres);   // the slot is free: the last round's MMAs are done
        // ---- natural tile -> round 0's operand (h / l), in place: one operand row per thread ----
        // lanes hold rows 0-4, whose tile bits 0-3 are the 16 contiguous coefficients of the tile:
        // the word loads of a warp hit distinct banks, the 16-byte chunk stores whole core matrices
        {
            const float *nat = reinterpret_cast<const float *>(AH);
            const float up = p.up;
            uint32_t tn0[3][4];
            digit_tables(p.natk, tn0);
            const uint32_t nb = xor_bits<8>(uint32_t(ttid), p.natrow);
            float x[64];
#pragma unroll
            for (int j = 0; j < 64; ++j) x[j] = nat[nb ^ tn0[0][j & 3] ^ tn0[1][(j >> 2) & 3] ^ tn0[2][j >> 4]];
            team_sync(team);
            const uint32_t o = row_off(ttid);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int e = 0; e < 8; e += 2)
                    split2(x[8 * c + e] * up, x[8 * c + e + 1] * up, hw[e >> 1], lw[e >> 1]);
                *reinterpret_cast<uint4 *>(AH + o + uint32_t(c) * kLBO) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(AL + o + uint32_t(c) * kLBO) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        }
        bool alive = true;
        for (int r = 0; r < p.nrounds; ++r) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            team_sync(team);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            bool issue = leader;
            if (leader && r >= p.nres) {     // a streamed image: wait for its bulk copy
                issue = mbar_wait(sbar, uphase);
                if (issue) {
                    uphase ^= 1;
                    u_pending = false;
                }                            // else no MMA and no commit: the team's wait below runs out
            }
            if (issue) {
                // The tensor pipe interleaves the two teams' MMAs when they are issued together, so
                // both finish together and the teams stay in step, each waiting for both teams' MMAs.
                // Team 1 holds its MMAs back (at most 20 us) while team 0's are in flight, which lets
                // one team's MMAs overlap the other team's epilogue instead.
                if (team == 0) {
                    pipe_busy = 1;
                } else {
                    const uint64_t t0 = tcg::global_ns();
                    while (pipe_busy && tcg::global_ns() - t0 < 20000) __nanosleep(64);
                }
                // D[:, 0:64] = h Uh^T and D[:, 64:128] = h Ul^T (one N = 128 chain over [Uh ; Ul]),
                // then D[:, 64:128] += l Uh^T (N = 64), for both M = 128 blocks
                const uint64_t ub = smem_desc(uslot(r));
#pragma unroll
                for (int mb = 0; mb < 2; ++mb) {
                    const uint32_t d = tmem + mb * 128;
#pragma unroll
                    for (int term = 0; term < 2; ++term) {
                        const uint32_t dd = d + (term == 0 ? 0u : 64u);
                        const uint64_t a = term == 0 ? adesc_h[mb] : adesc_l[mb];
                        const uint32_t idesc = term == 0 ? kIdesc128 : kIdesc64;
#pragma unroll
                        for (int ks = 0; ks < 4; ++ks) {
                            // a K step of 16 values is two core matrices (256 bytes): +16 in the
                            // descriptor's start-address field (address >> 4, bits 0-13)
                            const uint64_t da = a + uint64_t(ks * (2 * kLBO >> 4));
                            const uint64_t db = ub + uint64_t(ks * (2 * kLBO >> 4));
                            const uint32_t acc = (term | ks) ? 1u : 0u;
                            asm volatile(
                                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dd),
                                "l"(da), "l"(db), "r"(idesc), "r"(acc));
                        }
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
            }
            mma_pending = true;
            if (!team_and(mbar_wait(mbar, mphase), team)) {
                if (ttid == 0) atomicExch(status, 1);
                alive = false;
                break;
            }
            mphase ^= 1;
            mma_pending = false;
            if (team == 0 && leader) pipe_busy = 0;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const bool last = r + 1 == p.nrounds;
            if (leader && r >= p.nres && !last) stream_u(r + 1);   // this round's MMAs have read the slot
            if (last && leader && tn < p.ntiles) {
                // the slot's operands are consumed: the next tile's load (from L2) overlaps this epilogue
                int c[kMaxDims];
                tile_coords(p, tn, c);
                tcg::mbar_expect_tx(lbar, kSlotBytes);
                tma_load(&tmap, p.ndims, c, smem_u32(AH), lbar);
            }
            float v[64];
            tcg::tmem_ld32_pair_fma(taddr, taddr + 64, kLoScale, v);        // 2**11 x = 2**11 D1 + D2
            tcg::tmem_ld32_pair_fma(taddr + 32, taddr + 96, kLoScale, v + 32);
            if (!last) {
                // ---- epilogue: D -> the next round's operand (h / l) ----
                const Round &R = p.rounds[r];
                uint32_t tk[3][4];
                digit_tables(R.kc, tk);
                const uint32_t base = xor_bits<8>(uint32_t(ttid), R.rowc);
                store_all<true>(v, R.vec, base, tk, AH, AL);
            } else {
                // ---- last round: the row straight to global memory; lanes 0-15 cover 64 contiguous bytes ----
                int c[kMaxDims];
                tile_coords(p, t, c);
                int64_t rowg = tile_base(p, c);
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    if ((ttid >> i) & 1) rowg += p.lastg[i];
                float *row = st + rowg;
                const float down = p.down * kLoUnscale;
#pragma unroll
                for (int d2 = 0; d2 < 4; ++d2) {
                    const int64_t o2 = (d2 & 1 ? p.lastg[12] : 0) + (d2 & 2 ? p.lastg[13] : 0);
#pragma unroll
                    for (int d1 = 0; d1 < 4; ++d1) {
                        float *q = row + o2 + (d1 & 1 ? p.lastg[10] : 0) + (d1 & 2 ? p.lastg[11] : 0);
                        const int j = 4 * d1 + 16 * d2;
                        if (p.last_vec) {    // K digit 0 is local axis 0: four contiguous coefficients
                            *reinterpret_cast<float4 *>(q) =
                                make_float4(v[j] * down, v[j + 1] * down, v[j + 2] * down, v[j + 3] * down);
                        } else {
                            q[0] = v[j] * down;
                            q[p.lastg[8]] = v[j + 1] * down;
                            q[p.lastg[9]] = v[j + 2] * down;
                            q[p.lastg[8] + p.lastg[9]] = v[j + 3] * down;
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        }
        if (!alive) break;
        load_pending = tn < p.ntiles;
    }
    // ---- drain: the team's MMA and tile load in flight ----
    if (mma_pending) mbar_wait(mbar, mphase);
    if (load_pending) mbar_wait(lbar, lphase);
    if (!u_ok) mbar_wait(ubar, 0);
    if (u_pending) mbar_wait(sbar, uphase);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base_s), "n"(kTmemCols));
}

}  // namespace tma

}  // namespace dmg

using namespace dmg;

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

namespace {

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static std::once_flag once;
    static EncodeTiled fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
        (void)cudaGetLastError();
    });
    return fn;
}

}  // namespace

// Tensor-map dimensions of a pass (see the file comment); false when the
// resident digits need more than kMaxDims dimensions.
static bool tma_dims(int n, const int32_t *axes, tma::TmaPass &p, cuuint64_t *gdim, cuuint64_t *gstride_bytes,
                     cuuint32_t *box) {
    bool res[DM_MAX_QUBITS * 2] = {false};
    for (int r = 0; r < tc::kAxes; ++r) res[n - 1 - axes[r]] = true;   // digit position of each resident qubit
    int nd = 0, gap_first = 0;
    int pos = 0;
    while (pos < n) {
        if (!res[pos]) return false;   // only reached for position 0 (a chunk is always followed by its gap)
        int len = 0;
        while (pos + len < n && res[pos + len] && len < 4) ++len;
        int gap = 0;
        while (pos + len + gap < n && !res[pos + len + gap]) ++gap;
        if (nd == tma::kMaxDims) return false;
        p.box_log4[nd] = int8_t(len);
        p.gap_len[nd] = int8_t(gap);
        p.gap_first[nd] = int8_t(gap_first);
        p.start[nd] = int8_t(pos);
        gdim[nd] = cuuint64_t(1) << (2 * (len + gap));
        box[nd] = cuuint32_t(1) << (2 * len);
        if (nd > 0) gstride_bytes[nd - 1] = (cuuint64_t(1) << (2 * pos)) * sizeof(float);
        gap_first += gap;
        pos += len + gap;
        ++nd;
    }
    for (int i = nd; i < tma::kMaxDims; ++i) p.box_log4[i] = p.gap_len[i] = p.gap_first[i] = p.start[i] = 0;
    p.ndims = nd;
    return gap_first == n - tc::kAxes;
}

// Natural-tile tables: element offsets below 4**7, each a power of two (the TMA box is unswizzled).
static bool linear_tables(const uint32_t *rowc, const uint32_t *kc, int vec) {
    uint32_t seen = 0;
    for (int i = 0; i < 14; ++i) {
        const uint32_t c = i < 8 ? rowc[i] : kc[i - 8];
        if (c == 0 || (c & (c - 1)) || c >= uint32_t(tc::kTile) || (seen & c)) return false;
        seen |= c;
    }
    if (vec >= 0) {
        if (vec > 2 || kc[2 * vec] != 1 || kc[2 * vec + 1] != 2) return false;
    }
    return true;
}

// Operand tables: distinct powers of two inside one 32 KB image, 8-byte aligned
// apart from the vector digit's two bits.
static bool operand_tables(const uint32_t *rowc, const uint32_t *kc, int vec) {
    uint32_t seen = 0;
    for (int i = 0; i < 14; ++i) {
        const uint32_t c = i < 8 ? rowc[i] : kc[i - 8];
        if (c == 0 || (c & (c - 1)) || c >= tc::kABytes || (seen & c)) return false;
        seen |= c;
    }
    if (vec >= 0) {
        if (vec > 2 || kc[2 * vec] != 2 || kc[2 * vec + 1] != 4) return false;
        for (int i = 0; i < 14; ++i) {
            if (i >= 8 && (i - 8) / 2 == vec) continue;
            const uint32_t c = i < 8 ? rowc[i] : kc[i - 8];
            if (c % 8) return false;
        }
    }
    return true;
}

extern "C" int dm_apply_pass_tma(void *state_dev, int n, const dm_tc_pass *pass, const uint16_t *umats_dev,
                                 size_t umats_count, int *status_dev, void *stream) {
    DM_CHECK_ARG(state_dev && pass && umats_dev && status_dev && valid_n(n));
    if (reinterpret_cast<uintptr_t>(state_dev) & 15 || reinterpret_cast<uintptr_t>(umats_dev) & 15) return DM_ERR_ARG;
    if (n < tc::kAxes) return DM_ERR_PROGRAM;
    const int nr = pass->nrounds;
    if (nr < 1 || nr > tma::kMaxRounds) return DM_ERR_PROGRAM;
    for (int r = 0; r < tc::kAxes; ++r) {
        const int q = pass->axes[r];
        if (q < 0 || q >= n || (r > 0 && q >= pass->axes[r - 1])) return DM_ERR_PROGRAM;
    }
    if (pass->axes[0] != n - 1) return DM_ERR_PROGRAM;   // the contiguous axis is resident
    tma::TmaPass p{};
    cuuint64_t gdim[tma::kMaxDims], gstride[tma::kMaxDims];
    cuuint32_t box[tma::kMaxDims], estride[tma::kMaxDims];
    if (!tma_dims(n, pass->axes, p, gdim, gstride, box)) return DM_ERR_PROGRAM;
    p.nrounds = nr;
    p.nres = nr <= tma::kUSlots ? nr : tma::kStreamFrom;
    p.up = float(ldexp(1.0, n));
    p.down = float(ldexp(1.0, -n));
    p.ntiles = int64_t(1) << (2 * (n - tc::kAxes));
    if (!linear_tables(pass->natrow, pass->natk, -1)) return DM_ERR_PROGRAM;
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
        const bool ok = r + 1 == nr ? linear_tables(in.rowc, in.kc, -1) : operand_tables(in.rowc, in.kc, in.vec);
        if (!ok) return DM_ERR_PROGRAM;
        if (r + 1 == nr) {
            // the last round stores to global memory: tile bit b = bit b % 2 of local axis b / 2's digit
            for (int i = 0; i < 14; ++i) {
                const uint32_t c = i < 8 ? in.rowc[i] : in.kc[i - 8];
                int b = 0;
                while ((1u << b) != c) ++b;
                const int pos = n - 1 - pass->axes[b >> 1];
                p.lastg[i] = (int64_t(1) << (b & 1)) << (2 * pos);
            }
            // K digit 0 = local axis 0 (K bits 0, 1 at offsets 1, 2): every other bit is a multiple of
            // 4 elements, so each group of four lands 16-byte aligned
            p.last_vec = p.lastg[8] == 1 && p.lastg[9] == 2;
        }
        for (int i = 0; i < 8; ++i) o.rowc[i] = in.rowc[i];
        for (int i = 0; i < 6; ++i) o.kc[i] = in.kc[i];
        if (in.umoff < 0 || (in.umoff & 7) || size_t(in.umoff) + tma::kUHalves > umats_count) return DM_ERR_PROGRAM;
        o.umoff = in.umoff;
        p.uoff[r] = in.umoff;
    }
    EncodeTiled enc = encode_fn();
    if (!enc) return DM_ERR_CUDA;
    for (int i = 0; i < tma::kMaxDims; ++i) estride[i] = 1;
    CUtensorMap map;
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, cuuint32_t(p.ndims), state_dev, gdim, gstride, box, estride,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return DM_ERR_CUDA;
    const int64_t grid = std::min<int64_t>(sm_count(), (p.ntiles + tma::kTeams - 1) / tma::kTeams);
    if (ensure_max_dynamic_smem(reinterpret_cast<const void *>(tma::pass_tma_kernel), int(tma::kSmemBytes)) !=
        cudaSuccess)
        return DM_ERR_CUDA;
    tma::pass_tma_kernel<<<int(grid), tma::kThreads, tma::kSmemBytes, as_stream(stream)>>>(
        map, p, static_cast<float *>(state_dev), umats_dev, status_dev);
    count_launch();
    return launch_status();
}

// ---------------------------------------------------------------------------
// bounded-wait self-test: the failure path of every tensor-core kernel's waits
// ---------------------------------------------------------------------------

namespace dmg {
namespace tma {

// One thread waits, with a limit of limit_ns, on an mbarrier that nothing arrives on, as the
// pass kernels wait for an MMA commit or a tile load; the wait gives up and the kernel reports
// status 1, exactly as a pass kernel does before it drains and returns.
__global__ void wait_selftest_kernel(int *status, int64_t limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = smem_u32(&bar);
    tcg::mbar_init(b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (!tcg::mbar_wait(b, 0, uint64_t(limit_ns))) atomicExch(status, 1);
}

}  // namespace tma
}  // namespace dmg

extern "C" int dm_tc_wait_selftest(int *status_dev, int64_t limit_ns, void *stream) {
    DM_CHECK_ARG(status_dev && limit_ns > 0 && limit_ns <= 100000000);   // at most 0.1 s
    dmg::tma::wait_selftest_kernel<<<1, 1, 0, as_stream(stream)>>>(status_dev, limit_ns);
    count_launch();
    return launch_status();
}
