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

// ---------------------------------------------------------------------------
// template sweeps: an operation's coefficients composed from its recipe chain
// ---------------------------------------------------------------------------

constexpr int kCoefStride = 16;   // shared-memory coefficients per slot

// m <- (rotation about `axis` by angle, error (e0, e1)) * m, rows k0 / k1 only.
__device__ __forceinline__ void rot_apply(double (&m)[16], int axis, double angle, double e0, double e1) {
    // planes of rx, ry, rz: (Y, Z), (Z, X), (X, Y)  (basicaertools.py:106-124)
    const int k0 = axis == 0 ? 2 : axis == 1 ? 3 : 1;
    const int k1 = axis == 0 ? 3 : axis == 1 ? 1 : 2;
    double sn, cs;
    sincos(angle + e1, &sn, &cs);
    const double c = e0 * cs, s = e0 * sn;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const double a = m[4 * k0 + j], b = m[4 * k1 + j];
        m[4 * k0 + j] = c * a - s * b;
        m[4 * k1 + j] = s * a + c * b;
    }
}

// m <- memory noise (f, p, g) * m: X, Y rows scaled by sqrt(g) f; Z <- g Z + (1 - g)(2p - 1) I.
__device__ __forceinline__ void noise_apply(double (&m)[16], double f, double p, double g) {
    const double k = sqrt(g) * f, d = (1 - g) * (2 * p - 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        m[4 + j] *= k;
        m[8 + j] *= k;
        m[12 + j] = g * m[12 + j] + d * m[j];
    }
}

template <typename T>
__device__ void compose_slot(const dm_param_program &P, int slot, const double *prm, T *out) {
    const dm_param_slot sl = P.slots[slot];
    const dm_recipe &first = P.recipes[P.chain[sl.begin]];
    if (first.kind == DM_RECIPE_CX) {
        const double cav = prm[9], mean = prm[10];
        const double c2av = 4 * cav - 3;
        double sn, cs, sn2, cs2;
        sincos(mean, &sn, &cs);
        sincos(2 * mean, &sn2, &cs2);
        out[0] = T(cav * cs);
        out[1] = T(cav * sn);
        out[2] = T(0.5 * (1 + c2av * cs2));
        out[3] = T(0.5 * (1 - c2av * cs2));
        out[4] = T(c2av * sn * cs);
        return;
    }
    double m[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0 : 0.0;
    for (int c = 0; c < sl.len; ++c) {
        const dm_recipe &rc = P.recipes[P.chain[sl.begin + c]];
        if (rc.kind == DM_RECIPE_ROT) {
            for (int k = 0; k < rc.nrot; ++k) {
                const int ax = rc.axis[k];
                rot_apply(m, ax, rc.angle[k], prm[3 + 2 * ax], prm[4 + 2 * ax]);
            }
        } else if (rc.kind == DM_RECIPE_NOISE) {
            noise_apply(m, prm[0], prm[1], prm[2]);
        } else {   // DM_RECIPE_CONST: m <- C m (a diagonal pair map is a chain of one)
            const double *cm = P.consts + rc.const_off;
            if (sl.len == 1) {
#pragma unroll
                for (int i = 0; i < 16; ++i) m[i] = cm[i];
            } else {
                double t[16];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        t[4 * i + j] = cm[4 * i] * m[j] + cm[4 * i + 1] * m[4 + j] + cm[4 * i + 2] * m[8 + j] +
                                       cm[4 * i + 3] * m[12 + j];
#pragma unroll
                for (int i = 0; i < 16; ++i) m[i] = t[i];
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) out[i] = T(m[i]);
}

// Host check of a template program's recipes, chains and slots: slot s is op
// s of the concatenated passes (npasses of them; nops(p) ops in pass p, op o
// of kind op_kind(p, o)), and every slot's recipe chain must fit its op.
template <typename NOps, typename OpKind>
inline int validate_param_slots(const dm_param_program &P, int npasses, NOps nops, OpKind op_kind) {
    if (P.nslots < 0 || P.nchain < 0 || P.nrecipes < 0 || P.nconsts < 0) return DM_ERR_PROGRAM;
    if ((P.nslots && !P.slots) || (P.nchain && !P.chain) || (P.nrecipes && !P.recipes) || (P.nconsts && !P.consts))
        return DM_ERR_ARG;
    for (int r = 0; r < P.nrecipes; ++r) {
        const dm_recipe &rc = P.recipes[r];
        if (rc.kind == DM_RECIPE_ROT) {
            if (rc.nrot < 1 || rc.nrot > 3) return DM_ERR_PROGRAM;
            for (int k = 0; k < rc.nrot; ++k)
                if (rc.axis[k] < 0 || rc.axis[k] > 2) return DM_ERR_PROGRAM;
        } else if (rc.kind == DM_RECIPE_CONST) {
            if (rc.const_off < 0 || int64_t(rc.const_off) + 16 > P.nconsts) return DM_ERR_PROGRAM;
        } else if (rc.kind != DM_RECIPE_NOISE && rc.kind != DM_RECIPE_CX) {
            return DM_ERR_PROGRAM;
        }
    }
    for (int c = 0; c < P.nchain; ++c)
        if (P.chain[c] < 0 || P.chain[c] >= P.nrecipes) return DM_ERR_PROGRAM;
    int slot = 0;
    for (int p = 0; p < npasses; ++p) {
        for (int o = 0; o < nops(p); ++o, ++slot) {
            if (slot >= P.nslots) return DM_ERR_PROGRAM;
            const dm_param_slot sl = P.slots[slot];
            if (sl.len < 1 || sl.begin < 0 || int64_t(sl.begin) + sl.len > P.nchain) return DM_ERR_PROGRAM;
            const int kind = op_kind(p, o);
            for (int c = 0; c < sl.len; ++c) {
                const int rk = P.recipes[P.chain[sl.begin + c]].kind;
                const bool ok = kind == DM_OP_MAP1 ? (rk != DM_RECIPE_CX)
                                                   : (sl.len == 1 && rk == (kind == DM_OP_CX ? DM_RECIPE_CX
                                                                                             : DM_RECIPE_CONST));
                if (!ok) return DM_ERR_PROGRAM;
            }
        }
    }
    return slot == P.nslots ? DM_OK : DM_ERR_PROGRAM;
}

}  // namespace dmg
