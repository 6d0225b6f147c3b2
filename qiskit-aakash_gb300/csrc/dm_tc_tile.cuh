// Tile geometry and epilogue helpers shared by the tensor-core pass kernels
// (dm_tc.cu: cp.async-fed pass and batched sweeps; dm_tma.cu: TMA-fed pass).
//
// A tile holds the 4**7 = 16,384 coefficients that differ only in a pass's 7
// resident axes.  A round views it as a 256 x 64 FP16 operand (one row per
// group of the round's 3 axes) in the K-major core-matrix layout below, and
// the epilogue of each round writes the next round's operand (or, after the
// last round, the natural FP32 tile) through per-bit XOR offset tables.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "dm_gb300.h"
#include "dm_tcgen05.cuh"

namespace dmg {
namespace tc {

constexpr int kAxes = 7;                       // resident axes per tile
constexpr int kTile = 1 << (2 * kAxes);        // 16384 coefficients
constexpr int kGroups = kTile / 64;            // 256 rows per round
constexpr uint32_t kABytes = kGroups * 64 * 2; // 32 KB per FP16 operand image
constexpr uint32_t kBImage = 64 * 64 * 2;      // 8 KB per FP16 matrix image
constexpr float kLoScale = 2048.0f, kLoUnscale = 1.0f / 2048.0f;

// K-major core-matrix layout (no swizzle) of a rows x 64 FP16 operand: element
// (row, k) lives at byte (row%8)*16 + (k%8)*2 + (k/8)*128 + (row/8)*1024.
// LBO (next 16-byte core matrix along K) = 128 B, SBO (next 8 rows) = 1024 B.
constexpr uint32_t kLBO = 128, kSBO = 1024;

__device__ __forceinline__ uint32_t row_off(int row) { return (row & 7) * 16 + (row >> 3) * kSBO; }
__device__ __forceinline__ uint32_t k_off(int k) { return (k & 7) * 2 + (k >> 3) * kLBO; }

using tcg::cp_async16;
using tcg::cp_async_commit;
using tcg::cp_async_wait_all;
using tcg::mbar_wait;
using tcg::smem_u32;

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) { return tcg::smem_desc(saddr, kLBO, kSBO); }

// kind::f16, D = F32 (bits 4-5 = 1), A = B = F16 (bits 7-9, 10-12 = 0), both K-major, M = 128, N = 128 / 64.
constexpr uint32_t kIdesc128 = (1u << 4) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
constexpr uint32_t kIdesc64 = (1u << 4) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

struct Round {
    int8_t digits[3];
    int8_t vec;
    int32_t umoff;
    uint32_t rowc[8];
    uint32_t kc[6];
};

// XOR-combination of the offsets of the set bits of x (nbits of them).
template <int NB>
__device__ __forceinline__ uint32_t xor_bits(uint32_t x, const uint32_t *c) {
    uint32_t o = 0;
#pragma unroll
    for (int i = 0; i < NB; ++i)
        if ((x >> i) & 1) o ^= c[i];
    return o;
}

// Per-digit XOR tables of the 64 K indices: k -> t0[d0] ^ t1[d1] ^ t2[d2].
__device__ __forceinline__ void digit_tables(const uint32_t *kc, uint32_t (&t)[3][4]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        t[d][0] = 0;
        t[d][1] = kc[2 * d];
        t[d][2] = kc[2 * d + 1];
        t[d][3] = kc[2 * d] ^ kc[2 * d + 1];
    }
}

// x -> (h, l): h = fp16(x), l = fp16(2**11 (x - h)), two values at once with packed conversions
// (h2 = (fp16(a), fp16(b)) as FP16 bit patterns, l2 likewise)
__device__ __forceinline__ void split2(float a, float b, uint32_t &h2, uint32_t &l2) {
    const __half2 hh = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(hh);
    const __half2 ll = __floats2half2_rn((a - hf.x) * kLoScale, (b - hf.y) * kLoScale);
    h2 = *reinterpret_cast<const uint32_t *>(&hh);
    l2 = *reinterpret_cast<const uint32_t *>(&ll);
}

// The same split of accumulator values a = 2**11 x: h = fp16(2**-11 a) and
// l = fp16(a - 2**11 h), one FMA, exact (a - 2**11 h = 2**11 (x - h) is an
// FP32 number), so the result equals split2(2**-11 a, 2**-11 b) bit for bit.
__device__ __forceinline__ void split2_acc(float a, float b, uint32_t &h2, uint32_t &l2) {
    const __half2 hh = __floats2half2_rn(a * kLoUnscale, b * kLoUnscale);
    const float2 hf = __half22float2(hh);
    const __half2 ll = __floats2half2_rn(fmaf(-kLoScale, hf.x, a), fmaf(-kLoScale, hf.y, b));
    h2 = *reinterpret_cast<const uint32_t *>(&hh);
    l2 = *reinterpret_cast<const uint32_t *>(&ll);
}

// four accumulator values adjacent in K: one 64-bit store into each image
__device__ __forceinline__ void put_split4(unsigned char *AH, unsigned char *AL, uint32_t o, float a, float b,
                                           float c, float d) {
    uint32_t h0, l0, h1, l1;
    split2_acc(a, b, h0, l0);
    split2_acc(c, d, h1, l1);
    *reinterpret_cast<uint2 *>(AH + o) = make_uint2(h0, h1);
    *reinterpret_cast<uint2 *>(AL + o) = make_uint2(l0, l1);
}

// Epilogue stores of one thread's 64 values (K index j = d0 + 4 d1 + 16 d2)
// at base ^ t[0][d0] ^ t[1][d1] ^ t[2][d2].  With a vector digit D the four
// values along D are adjacent in the destination: one 64-bit store per
// FP16 image (SPLIT), or one 128-bit FP32 store into the natural tile.
template <int D, bool SPLIT>
__device__ __forceinline__ void store_vec(const float (&v)[64], uint32_t base, const uint32_t (&t)[3][4],
                                          unsigned char *AH, unsigned char *AL) {
    constexpr int S = 1 << (2 * D);
    constexpr int X = D == 0 ? 1 : 0, Y = D == 2 ? 1 : 2;   // the two other digits
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const int j0 = (x << (2 * X)) | (y << (2 * Y));
            const uint32_t o = base ^ t[X][x] ^ t[Y][y];
            if (SPLIT)
                put_split4(AH, AL, o, v[j0], v[j0 + S], v[j0 + 2 * S], v[j0 + 3 * S]);
            else
                *reinterpret_cast<float4 *>(AH + 4 * o) = make_float4(v[j0], v[j0 + S], v[j0 + 2 * S], v[j0 + 3 * S]);
        }
}

template <bool SPLIT>
__device__ __forceinline__ void store_all(const float (&v)[64], int vec, uint32_t base, const uint32_t (&t)[3][4],
                                          unsigned char *AH, unsigned char *AL) {
    if (vec == 0) {
        store_vec<0, SPLIT>(v, base, t, AH, AL);
    } else if (vec == 1) {
        store_vec<1, SPLIT>(v, base, t, AH, AL);
    } else if (vec == 2) {
        store_vec<2, SPLIT>(v, base, t, AH, AL);
    } else if (SPLIT) {
#pragma unroll
        for (int j = 0; j < 64; j += 2) {   // conversions in pairs, 16-bit stores
            uint32_t h2, l2;
            split2_acc(v[j], v[j + 1], h2, l2);
            const uint32_t o0 = base ^ t[0][j & 3] ^ t[1][(j >> 2) & 3] ^ t[2][j >> 4];
            const uint32_t o1 = o0 ^ t[0][(j & 3) ^ 1] ^ t[0][j & 3];
            *reinterpret_cast<unsigned short *>(AH + o0) = (unsigned short)(h2 & 0xFFFFu);
            *reinterpret_cast<unsigned short *>(AL + o0) = (unsigned short)(l2 & 0xFFFFu);
            *reinterpret_cast<unsigned short *>(AH + o1) = (unsigned short)(h2 >> 16);
            *reinterpret_cast<unsigned short *>(AL + o1) = (unsigned short)(l2 >> 16);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            const uint32_t o = base ^ t[0][j & 3] ^ t[1][(j >> 2) & 3] ^ t[2][j >> 4];
            reinterpret_cast<float *>(AH)[o] = v[j];
        }
    }
}

}  // namespace tc
}  // namespace dmg
