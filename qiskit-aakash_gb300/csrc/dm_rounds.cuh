// Register-round operation bodies shared by the fused-pass kernels: a
// group of 4**R coefficients that differ only in R local axes ("digits")
// sits in registers, v[j] with j = d0 + 4 d1 + 16 d2, and the round's
// operations (4x4 maps on one digit, CX and diagonal pair maps on two) are
// applied to it in place.
#pragma once

#include "dm_common.cuh"

namespace dmg {

template <typename T>
struct CxCoef {
    T c, s, c2, s2, cs;
};

template <typename T>
__device__ __forceinline__ void map4(const T *m, bool row0_id, T &x0, T &x1, T &x2, T &x3) {
    T y0 = row0_id ? x0 : fma(m[0], x0, fma(m[1], x1, fma(m[2], x2, m[3] * x3)));
    T y1 = fma(m[4], x0, fma(m[5], x1, fma(m[6], x2, m[7] * x3)));
    T y2 = fma(m[8], x0, fma(m[9], x1, fma(m[10], x2, m[11] * x3)));
    T y3 = fma(m[12], x0, fma(m[13], x1, fma(m[14], x2, m[15] * x3)));
    x0 = y0;
    x1 = y1;
    x2 = y2;
    x3 = y3;
}

// x[4*pc + pt]: control Pauli pc, target Pauli pt.  basicaertools.py:346-363
// (the control > target branch, :371-388, is the same map in (control,
// target) coordinates).
template <typename T>
__device__ __forceinline__ void cx16(T *x, const CxCoef<T> &k, bool ideal) {
    if (ideal) {
        T t;
        t = x[2]; x[2] = x[14]; x[14] = t;          // IY <-> ZY
        t = x[3]; x[3] = x[15]; x[15] = t;          // IZ <-> ZZ
        t = x[4]; x[4] = x[5]; x[5] = t;            // XI <-> XX
        t = x[8]; x[8] = x[9]; x[9] = t;            // YI <-> YX
        T xy = x[6], xz = x[7], yy = x[10], yz = x[11];
        x[6] = yz;                                  // XY <-  YZ
        x[7] = -yy;                                 // XZ <- -YY
        x[10] = -xz;                                // YY <- -XZ
        x[11] = xy;                                 // YZ <-  XY
        return;
    }
    const T c = k.c, s = k.s, c2 = k.c2, s2 = k.s2, cs = k.cs;
    T i2 = x[2], i3 = x[3], z2 = x[14], z3 = x[15];
    T x0 = x[4], x1 = x[5], x2 = x[6], x3 = x[7];
    T y0 = x[8], y1 = x[9], y2 = x[10], y3 = x[11];
    T d3 = i3 - z3, d2 = i2 - z2;
    x[2] = fma(s2, i2, fma(c2, z2, -cs * d3));
    x[14] = fma(c2, i2, fma(s2, z2, cs * d3));
    x[3] = fma(s2, i3, fma(c2, z3, cs * d2));
    x[15] = fma(c2, i3, fma(s2, z3, -cs * d2));
    x[4] = fma(c, x1, -s * y0);
    x[5] = fma(c, x0, -s * y1);
    x[6] = fma(-s, y2, c * y3);
    x[7] = fma(-c, y2, -s * y3);
    x[8] = fma(s, x0, c * y1);
    x[9] = fma(s, x1, c * y0);
    x[10] = fma(s, x2, -c * x3);
    x[11] = fma(c, x2, s * x3);
}

// Register index j of a group holds round digits (j & 3, (j >> 2) & 3, j >> 4).
// The common trace-preserving map whose X and Y rows take no I component
// (gates, memory noise, measurements, resets): 10 FMAs per 4 values.
template <typename T>
__device__ __forceinline__ void map4_tp_xy(const T *m, T &x0, T &x1, T &x2, T &x3) {
    const T y1 = fma(m[5], x1, fma(m[6], x2, m[7] * x3));
    const T y2 = fma(m[9], x1, fma(m[10], x2, m[11] * x3));
    const T y3 = fma(m[12], x0, fma(m[13], x1, fma(m[14], x2, m[15] * x3)));
    x1 = y1;
    x2 = y2;
    x3 = y3;
}

template <typename T, int R, int D>
__device__ __forceinline__ void reg_map1(T (&v)[1 << (2 * R)], const T *__restrict__ mg, bool row0_id, bool xy_unital) {
    T m[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = mg[i];
    constexpr int S = 1 << (2 * D);
    if (row0_id && xy_unital) {
#pragma unroll
        for (int o = 0; o < (1 << (2 * (R - 1))); ++o) {
            const int j0 = ((o >> (2 * D)) << (2 * D + 2)) | (o & (S - 1));
            map4_tp_xy(m, v[j0], v[j0 + S], v[j0 + 2 * S], v[j0 + 3 * S]);
        }
        return;
    }
#pragma unroll
    for (int o = 0; o < (1 << (2 * (R - 1))); ++o) {
        const int j0 = ((o >> (2 * D)) << (2 * D + 2)) | (o & (S - 1));
        map4(m, row0_id, v[j0], v[j0 + S], v[j0 + 2 * S], v[j0 + 3 * S]);
    }
}

__host__ __device__ constexpr int ins0(int g, int pos) {
    return ((g >> (2 * pos)) << (2 * pos + 2)) | (g & ((1 << (2 * pos)) - 1));
}

// Register index of the (0, 0) entry of pair group o for round digits (DA, DB).
template <int DA, int DB>
__device__ __forceinline__ constexpr int pair_base(int o) {
    return ins0(ins0(o, DA < DB ? DA : DB), DA < DB ? DB : DA);
}

// CX on the registers of one pair group, in place.  Entry (pa, pb) of the
// group lives at v[j0 + pa*SA + pb*SB]; (pa, pb) = (control, target) Paulis.
template <typename T, int R, int J0, int SA, int SB>
__device__ __forceinline__ void reg_cx_group(T (&v)[1 << (2 * R)], const CxCoef<T> &k, bool ideal) {
#define DM_V(pa, pb) v[J0 + (pa) * SA + (pb) * SB]
    if (ideal) {
        T t;
        t = DM_V(0, 2); DM_V(0, 2) = DM_V(3, 2); DM_V(3, 2) = t;
        t = DM_V(0, 3); DM_V(0, 3) = DM_V(3, 3); DM_V(3, 3) = t;
        t = DM_V(1, 0); DM_V(1, 0) = DM_V(1, 1); DM_V(1, 1) = t;
        t = DM_V(2, 0); DM_V(2, 0) = DM_V(2, 1); DM_V(2, 1) = t;
        const T xy = DM_V(1, 2), xz = DM_V(1, 3), yy = DM_V(2, 2), yz = DM_V(2, 3);
        DM_V(1, 2) = yz;
        DM_V(1, 3) = -yy;
        DM_V(2, 2) = -xz;
        DM_V(2, 3) = xy;
    } else {
        const T c = k.c, s = k.s, c2 = k.c2, s2 = k.s2, cs = k.cs;
        const T i2 = DM_V(0, 2), i3 = DM_V(0, 3), z2 = DM_V(3, 2), z3 = DM_V(3, 3);
        const T x0 = DM_V(1, 0), x1 = DM_V(1, 1), x2 = DM_V(1, 2), x3 = DM_V(1, 3);
        const T y0 = DM_V(2, 0), y1 = DM_V(2, 1), y2 = DM_V(2, 2), y3 = DM_V(2, 3);
        const T d3 = i3 - z3, d2 = i2 - z2;
        DM_V(0, 2) = fma(s2, i2, fma(c2, z2, -cs * d3));
        DM_V(3, 2) = fma(c2, i2, fma(s2, z2, cs * d3));
        DM_V(0, 3) = fma(s2, i3, fma(c2, z3, cs * d2));
        DM_V(3, 3) = fma(c2, i3, fma(s2, z3, -cs * d2));
        DM_V(1, 0) = fma(c, x1, -s * y0);
        DM_V(1, 1) = fma(c, x0, -s * y1);
        DM_V(1, 2) = fma(-s, y2, c * y3);
        DM_V(1, 3) = fma(-c, y2, -s * y3);
        DM_V(2, 0) = fma(s, x0, c * y1);
        DM_V(2, 1) = fma(s, x1, c * y0);
        DM_V(2, 2) = fma(s, x2, -c * x3);
        DM_V(2, 3) = fma(c, x2, s * x3);
    }
#undef DM_V
}

template <typename T, int R, int DA, int DB, int O>
__device__ __forceinline__ void reg_diag_row(T (&v)[1 << (2 * R)], int pa, const T (&d)[4]) {
    constexpr int SA = 1 << (2 * DA), SB = 1 << (2 * DB);
    constexpr int J0 = pair_base<DA, DB>(O);
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (q == pa) {
#pragma unroll
            for (int pb = 0; pb < 4; ++pb) v[J0 + q * SA + pb * SB] *= d[pb];
        }
}

template <typename T, int R, int DA, int DB>
__device__ __forceinline__ void reg_pair(T (&v)[1 << (2 * R)], const dm_op &op, const T *__restrict__ mg) {
    constexpr int SA = 1 << (2 * DA), SB = 1 << (2 * DB);
    if (op.kind == DM_OP_CX) {
        const bool ideal = (op.flags & DM_CX_IDEAL) != 0;
        CxCoef<T> cx{T(1), T(0), T(1), T(0), T(0)};
        if (!ideal) {
            cx.c = mg[0];
            cx.s = mg[1];
            cx.c2 = mg[2];
            cx.s2 = mg[3];
            cx.cs = mg[4];
        }
        reg_cx_group<T, R, pair_base<DA, DB>(0), SA, SB>(v, cx, ideal);
        if constexpr (R > 2) {
            reg_cx_group<T, R, pair_base<DA, DB>(1), SA, SB>(v, cx, ideal);
            reg_cx_group<T, R, pair_base<DA, DB>(2), SA, SB>(v, cx, ideal);
            reg_cx_group<T, R, pair_base<DA, DB>(3), SA, SB>(v, cx, ideal);
        }
    } else {  // DM_OP_DIAG2: one row of four coefficients at a time
#pragma unroll
        for (int pa = 0; pa < 4; ++pa) {
            T d[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) d[i] = mg[4 * pa + i];
            reg_diag_row<T, R, DA, DB, 0>(v, pa, d);
            if constexpr (R > 2) {
                reg_diag_row<T, R, DA, DB, 1>(v, pa, d);
                reg_diag_row<T, R, DA, DB, 2>(v, pa, d);
                reg_diag_row<T, R, DA, DB, 3>(v, pa, d);
            }
        }
    }
}

// Digit positions of an op inside its round: flags bits 8-9 (axis a), 12-13 (axis b).
template <typename T, int R>
__device__ __forceinline__ void reg_apply(T (&v)[1 << (2 * R)], const dm_op &op, const T *__restrict__ mats) {
    const T *mg = mats + op.moff;
    const int da = (op.flags >> 8) & 3, db = (op.flags >> 12) & 3;
    if (op.kind == DM_OP_MAP1) {
        const bool row0 = (op.flags & DM_MAP1_ROW0_IDENTITY) != 0;
        const bool xy = (op.flags & DM_MAP1_XY_UNITAL) != 0;
        if (da == 0) reg_map1<T, R, 0>(v, mg, row0, xy);
        else if (da == 1) reg_map1<T, R, 1>(v, mg, row0, xy);
        else if constexpr (R > 2) reg_map1<T, R, 2>(v, mg, row0, xy);
        return;
    }
    if constexpr (R == 2) {
        if (da == 0) reg_pair<T, R, 0, 1>(v, op, mg);
        else reg_pair<T, R, 1, 0>(v, op, mg);
    } else {
        const int code = da * 4 + db;
        switch (code) {
            case 1: reg_pair<T, R, 0, 1>(v, op, mg); break;
            case 2: reg_pair<T, R, 0, 2>(v, op, mg); break;
            case 4: reg_pair<T, R, 1, 0>(v, op, mg); break;
            case 6: reg_pair<T, R, 1, 2>(v, op, mg); break;
            case 8: reg_pair<T, R, 2, 0>(v, op, mg); break;
            case 9: reg_pair<T, R, 2, 1>(v, op, mg); break;
            default: break;
        }
    }
}

}  // namespace dmg
