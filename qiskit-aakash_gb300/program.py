"""Pauli transfer matrices and the fused-pass planner.

Every gate, noise channel and measurement update of the reference acts on
one or two Pauli axes of the coefficient vector as a small real linear map:

* rotations Rz/Ry/Rx with the averaged-angle error model
  (basicaertools.py:93-126): a 4x4 map mixing two of X, Y, Z;
  U3 = Rz(lambda), Ry(theta), Rz(phi) applied in that order
  (basicaertools.py:69-90);
* memory noise (dm_simulator.py:397-425): X, Y scaled by sqrt(g) f and
  Z <- g Z + (1-g)(2p-1) I, a 4x4 map with an I->Z entry;
* X/Y/Z/N measurement updates (dm_simulator.py:574-704) and reset
  (:810-823): 4x4 projections;
* CX with the transition-selective-pulse error (basicaertools.py:310-392):
  a 16-entry map on the (control, target) pair, a signed permutation when
  ideal;
* the Bell-basis projection (dm_simulator.py:749-756): a diagonal 16-entry map.

The planner turns a run of such operations into fused passes: each pass
names up to ``kmax`` resident qubit axes (always including the lowest
``low`` axes, which are contiguous in memory) and the operations it applies
to every tile of those axes.  Operations on disjoint axes commute, so an
operation may run in an earlier pass than an operation that precedes it in
program order, provided every earlier operation sharing one of its axes
has run: the planner scans the pending operations in order and takes every
operation whose axes fit in the pass and none of whose axes is held back by
an earlier operation it could not take.  Consecutive 4x4 maps on one axis
inside a pass are multiplied together (in FP64) into one map.
"""
import functools
import math

import numpy as np

from . import _native as N

_ROT_PLANES = {'rz': (1, 2), 'ry': (3, 1), 'rx': (2, 3)}

IDENTITY4 = np.eye(4)


def rotation_ptm(axis, angle, err):
    """4x4 map of one rotation with error (<cos>, mean): basicaertools.py:106-124."""
    if axis not in _ROT_PLANES:
        from .exceptions import QiskitError
        raise QiskitError('Gate is not among the valid decomposition types: %s' % axis)
    c = err[0] * math.cos(angle + err[1])
    s = err[0] * math.sin(angle + err[1])
    k0, k1 = _ROT_PLANES[axis]
    m = np.eye(4)
    m[k0, k0] = c
    m[k0, k1] = -s
    m[k1, k1] = c
    m[k1, k0] = s
    return m


def rotations_ptm(gate, errors):
    """4x4 map of the rotations [(axis, angle), ...] applied in order, each with its axis's
    error (<cos>, mean) from ``errors`` (basicaertools.py:106-124): rotation_ptm(...) @ ... @ I
    composed on plain floats (a rotation mixes two rows), one array at the end."""
    m = [[1.0, 0.0, 0.0, 0.0], [0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0]]
    for axis, angle in gate:
        planes = _ROT_PLANES.get(axis)
        if planes is None:
            from .exceptions import QiskitError
            raise QiskitError('Gate is not among the valid decomposition types: %s' % axis)
        e0, e1 = errors[axis][0], errors[axis][1]
        c = e0 * math.cos(angle + e1)
        s = e0 * math.sin(angle + e1)
        k0, k1 = planes
        r0, r1 = m[k0], m[k1]
        m[k0] = [c * a - s * b for a, b in zip(r0, r1)]
        m[k1] = [s * a + c * b for a, b in zip(r0, r1)]
    return np.array(m)


def u_gate_ptm(name, params, rotation_error):
    """u1 / u3 as the product of its rotations (basicaertools.py:69-90)."""
    p = [float(x) for x in params]
    if name in ('U', 'u3'):
        seq = (('rz', p[2]), ('ry', p[0]), ('rz', p[1]))
    elif name == 'u1':
        seq = (('rz', p[0]),)
    else:
        from .exceptions import QiskitError
        raise QiskitError('Gate is not among the valid types: %s' % name)
    m = np.eye(4)
    for axis, ang in seq:
        m = rotation_ptm(axis, ang, rotation_error[axis]) @ m
    return m


def noise_ptm(f, p, g):
    """Per-qubit memory noise of one clock cycle (dm_simulator.py:408-422)."""
    k = math.sqrt(g) * f
    d = (1 - g) * (2 * p - 1)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0
    m[1, 1] = k
    m[2, 2] = k
    m[3, 3] = g
    m[3, 0] = d
    return m


def measure_ptm(basis, err, nvec=None):
    """State update of a single-qubit measurement (dm_simulator.py:574-704)."""
    m = np.zeros((4, 4))
    m[0, 0] = 1.0
    if basis == 'X':
        m[1, 1] = err
    elif basis == 'Y':
        m[2, 2] = err
    elif basis == 'Z':
        m[3, 3] = err
    elif basis == 'N':
        v = [float(x) for x in nvec]
        for r in range(3):
            for c in range(3):
                m[r + 1, c + 1] = err * v[r] * v[c]
    else:
        raise ValueError(basis)
    return m


def reset_ptm():
    """Reset to |0>: X, Y <- 0, Z <- I (dm_simulator.py:810-823)."""
    m = np.zeros((4, 4))
    m[0, 0] = 1.0
    m[3, 0] = 1.0
    return m


def cx_coefficients(tsp):
    """(c, s, c2, s2, cs) of the noisy CX, basicaertools.py:329-336, and whether it is ideal."""
    cav, mean = float(tsp[0]), float(tsp[1])
    c2av = 4 * cav - 3
    coef = (cav * math.cos(mean), cav * math.sin(mean),
            0.5 * (1 + c2av * math.cos(2 * mean)), 0.5 * (1 - c2av * math.cos(2 * mean)),
            c2av * math.sin(mean) * math.cos(mean))
    ideal = coef == (1.0, 0.0, 1.0, 0.0, 0.0)
    return coef, ideal


def bell_projection_diag(err):
    """Diagonal of the Bell-measurement update on (slower axis, faster axis), index 4*i + j."""
    d = np.zeros(16)
    d[0] = 1.0
    for i in (1, 2, 3):
        d[5 * i] = err
    return d


# ---------------------------------------------------------------------------
# operations
# ---------------------------------------------------------------------------

class Op:
    """One pending operation: kind in {'map1', 'cx', 'diag2', 'map2'}; axes are qubits.

    ``src`` lists the indices (in the planner's input) of the operations this
    one stands for: a composed 4x4 map lists the maps it multiplies, in
    application order.  Batched programs use it to rebuild the coefficients
    of a shared plan for each instance.  ``tag`` names where a 4x4 map came
    from (('rot', rotations) for a gate, ('noise',) for memory noise), so a
    template program can recompute it from an instance's noise parameters.
    """
    __slots__ = ('kind', 'axes', 'data', 'ideal', 'src', 'tag')

    def __init__(self, kind, axes, data, ideal=False, src=None, tag=None):
        self.kind = kind
        self.axes = tuple(axes)
        self.data = data
        self.ideal = ideal
        self.src = src
        self.tag = tag

    def __repr__(self):
        return 'Op(%s, %s)' % (self.kind, self.axes)


class Pass:
    """A planned pass: resident qubits (decreasing) and ops with local axes."""
    __slots__ = ('axes', 'ops')

    def __init__(self, axes, ops):
        self.axes = axes
        self.ops = ops

    def local(self, q):
        return self.axes.index(q)


def plan_passes(ops, n, kmax, low, partial=False):
    """Group ``ops`` (program order) into fused passes.

    Returns a list of Pass; each pass's op list preserves program order
    among the ops it holds, and per axis the ops of successive passes are
    consecutive runs of that axis's ops, so applying the passes in order
    equals applying ``ops`` in order.

    With ``partial`` the ops are a prefix of a longer stream: only the
    passes whose scan closed before the end of ``ops`` are returned (they
    are exactly the passes the whole stream would give), together with the
    ops they left, in order: ``(passes, rest)``.
    """
    kmax = min(kmax, n)
    low = min(low, kmax)
    base = tuple(range(n - 1, n - 1 - low, -1))
    pending = list(ops)
    index_of = {id(op): i for i, op in enumerate(pending)}
    passes = []
    while pending:
        resident = set(base)
        full = len(resident) >= kmax
        blocked = set()
        closed = False
        taken_idx = []
        body = []          # list of Op (possibly composed)
        last_on_axis = {}  # axis -> index into body of the last op touching it
        for i, op in enumerate(pending):
            axes = op.axes
            if blocked.intersection(axes) or \
                    len(resident) + sum(a not in resident for a in axes) > kmax or \
                    len(body) >= N.DM_MAX_PASS_OPS:
                blocked.update(axes)
                # Once the pass is full and every resident axis is held back,
                # no later operation can be taken.
                if (full and blocked.issuperset(resident)) or len(blocked) >= n:
                    closed = True
                    break
                continue
            grow = [a for a in axes if a not in resident]
            resident.update(grow)
            taken_idx.append(i)
            src = op.src if op.src is not None else [index_of[id(op)]]
            if op.kind == 'map1':
                a = axes[0]
                j = last_on_axis.get(a)
                if j is not None and body[j].kind == 'map1':
                    body[j] = Op('map1', (a,), op.data @ body[j].data, src=body[j].src + src)
                    continue
                body.append(Op('map1', axes, op.data, src=src))
            else:
                body.append(Op(op.kind, axes, op.data, op.ideal, src=src))
            for a in axes:
                last_on_axis[a] = len(body) - 1
            if len(resident) >= kmax:
                full = True
        if not taken_idx:
            raise RuntimeError('planner made no progress')
        if partial and not closed:
            return passes, pending     # later ops could still join this pass
        keep = set(taken_idx)
        pending = [op for i, op in enumerate(pending) if i not in keep]
        axes = sorted(resident, reverse=True)
        passes.append(Pass(axes, body))
    return (passes, []) if partial else passes


def plan_rounds(p, width, pad='low'):
    """Group a pass's ops into register rounds of ``width`` local axes.

    Returns a list of (axes, ops): ``axes`` the round's local axes (ascending,
    exactly ``width`` of them, padded with untouched axes), ``ops`` the ops
    (axes in local numbering) in the order they run.  Built with the same
    dependency-respecting scan as the passes themselves, over the tile's
    local axes with no mandatory axes.
    """
    k = len(p.axes)
    local = [Op(op.kind, tuple(p.local(a) for a in op.axes), op.data, op.ideal, src=op.src) for op in p.ops]
    planned = plan_passes(local, k, width, 0)
    rounds = []
    for i, r in enumerate(planned):
        axes = sorted(r.axes)
        # 'low': pad with the lowest axes (axis 0 in a round lets the CUDA-core kernel move
        # 16-byte vectors); 'neighbors': first the axes the next round uses (its epilogue input
        # then shares them, so the tensor-core epilogue stores whole vectors), then the previous
        # round's
        nxt = sorted(planned[i + 1].axes) if i + 1 < len(planned) and pad == 'neighbors' else []
        prv = rounds[-1][0] if rounds and pad == 'neighbors' else []
        if pad == 'neighbors' and i == 0:
            nxt = [0] + nxt      # round 0 reads the natural tile: axis 0 gives 16-byte loads
        for a in nxt + prv + list(range(k)):
            if len(axes) >= width:
                break
            if a not in axes:
                axes.append(a)
        rounds.append((sorted(axes), r.ops))
    return rounds


# Largest pass (resident axes) the pipelined round kernel holds per dtype.
ROUND_MAX_AXES = {np.dtype(np.float32): 7, np.dtype(np.float64): 6}


def encode_pass(p, mats, dtype_np, round_width=None, n=None):
    """Fill a ctypes DmPass for ``p``; append its coefficients to ``mats`` (list of arrays).

    With ``round_width`` (and the register count ``n``) the ops are grouped
    into register rounds when the pipelined round kernel can run the pass:
    at least ``round_width`` and at most ROUND_MAX_AXES resident axes, the
    lowest qubit axis resident (16-byte chunks are contiguous), no 16x16
    general maps, and the rounds fit the descriptor.
    """
    dp = N.DmPass()
    dp.k = len(p.axes)
    for r, q in enumerate(p.axes):
        dp.axes[r] = q
    rounds = None
    if round_width and n is not None and round_width <= dp.k <= ROUND_MAX_AXES[np.dtype(dtype_np)] \
            and p.axes[0] == n - 1 and all(op.kind != 'map2' for op in p.ops):
        rounds = plan_rounds(p, round_width)
        if len(rounds) > N.DM_MAX_ROUNDS or sum(len(ops) for _, ops in rounds) > N.DM_MAX_PASS_OPS:
            rounds = None
    if rounds is not None:
        ops_local = []
        dp.nrounds = len(rounds)
        for ri, (axes, rops) in enumerate(rounds):
            for i, a in enumerate(axes):
                dp.round_axes[ri][i] = a
            for i in range(len(axes), 4):
                dp.round_axes[ri][i] = -1
            for op in rops:
                ops_local.append((op, [axes.index(a) for a in op.axes]))
            dp.round_end[ri] = len(ops_local)
    else:
        dp.nrounds = 0
        ops_local = [(Op(op.kind, tuple(p.local(a) for a in op.axes), op.data, op.ideal), None) for op in p.ops]
    dp.nops = len(ops_local)
    off = sum(m.size for m in mats)
    for i, (op, digits) in enumerate(ops_local):
        o = dp.ops[i]
        o.a = op.axes[0]
        o.moff = off
        if op.kind == 'map1':
            o.kind = N.DM_OP_MAP1
            m = np.ascontiguousarray(op.data, dtype=np.float64).reshape(16)
            flags = N.DM_MAP1_ROW0_IDENTITY if (m[0] == 1.0 and not m[1:4].any()) else 0
            flags |= N.DM_MAP1_XY_UNITAL if (m[4] == 0.0 and m[8] == 0.0) else 0
            o.b = 0
        elif op.kind == 'cx':
            o.kind = N.DM_OP_CX
            o.b = op.axes[1]
            flags = N.DM_CX_IDEAL if op.ideal else 0
            m = np.asarray(op.data, dtype=np.float64)
        elif op.kind == 'diag2':
            o.kind = N.DM_OP_DIAG2
            o.b = op.axes[1]
            flags = 0
            m = np.asarray(op.data, dtype=np.float64).reshape(16)
        elif op.kind == 'map2':
            o.kind = N.DM_OP_MAP2
            o.b = op.axes[1]
            flags = 0
            m = np.asarray(op.data, dtype=np.float64).reshape(256)
        else:
            raise ValueError(op.kind)
        if digits is not None:              # round digit positions of the op's axes
            flags |= digits[0] << 8
            if len(digits) > 1:
                flags |= digits[1] << 12
        o.flags = flags
        mats.append(m.astype(dtype_np))
        off += m.size
    return dp


# ---------------------------------------------------------------------------
# tensor-core rounds
# ---------------------------------------------------------------------------

TC_AXES = 7   # resident axes of a tensor-core pass (tiles of 4**7 FP32 coefficients)


class TcPlanError(RuntimeError):
    """A pass that does not fit a tensor-core descriptor (more rounds than DM_MAX_ROUNDS)."""


class OpTableError(TcPlanError):
    """A tensor-core pass with more ops than a DmBatchPass holds (its rounds fit; the host composes them)."""

# digits (d0, d1, d2) of the 64 round indices j = d0 + 4 d1 + 16 d2
_J = np.arange(64)
_DIG = np.stack([_J & 3, (_J >> 2) & 3, _J >> 4])


def _with_digit(d, pos, val):
    out = d.copy()
    out[pos] = val
    return out[0] + 4 * out[1] + 16 * out[2]


def op_matrix64(op, axes3):
    """64x64 map of one op on the round index j (digit i <-> local axis axes3[i])."""
    M = np.zeros((64, 64))
    if op.kind == 'map1':
        d = axes3.index(op.axes[0])
        src = _DIG[d]
        for p in range(4):
            M[_with_digit(_DIG, d, p), _J] += op.data[p, src]
        return M
    da, db = axes3.index(op.axes[0]), axes3.index(op.axes[1])
    if op.kind == 'cx':
        m16 = cx_matrix16(op.data, op.ideal)
    elif op.kind == 'diag2':
        m16 = np.diag(op.data)
    else:
        m16 = np.asarray(op.data)
    src = 4 * _DIG[da] + _DIG[db]
    for dst in range(16):
        w = m16[dst, src]
        nz = w != 0
        d2 = _DIG.copy()
        d2[da] = dst >> 2
        d2[db] = dst & 3
        M[(d2[0] + 4 * d2[1] + 16 * d2[2])[nz], _J[nz]] += w[nz]
    return M


def cx_matrix16(coef, ideal):
    """The CX transfer matrix on (control, target) Paulis, index 4*pc + pt (basicaertools.py:346-363)."""
    c, s, c2, s2, cs = (1.0, 0.0, 1.0, 0.0, 0.0) if ideal else coef
    M = np.eye(16)
    rows = {
        2: {2: s2, 14: c2, 3: -cs, 15: cs}, 14: {2: c2, 14: s2, 3: cs, 15: -cs},
        3: {3: s2, 15: c2, 2: cs, 14: -cs}, 15: {3: c2, 15: s2, 2: -cs, 14: cs},
        4: {5: c, 8: -s}, 5: {4: c, 9: -s}, 6: {10: -s, 11: c}, 7: {10: -c, 11: -s},
        8: {4: s, 9: c}, 9: {5: s, 8: c}, 10: {6: s, 7: -c}, 11: {6: c, 7: s},
    }
    for r, ent in rows.items():
        M[r, :] = 0
        for col, v in ent.items():
            M[r, col] = v
    return M


# FP16 3-split of the tensor-core rounds.  Inside a pass the tile is held in
# scaled units x' = 2**n a (|x'| <= 1 for a physical state), split as
# x' = h + 2**-11 l with h = fp16(x'), l = fp16(2**11 (x' - h)); the round
# matrix likewise U = Uh + 2**-11 Ul.  Two FP32 accumulators collect
#     h (2**11 Uh)^T   and   h Ul^T + l Uh^T,
# whose sum is 2**11 (x' U^T) + O(2**-22); the epilogue adds them and
# multiplies by 2**-11 (exact).
TC_LO_SCALE = 2048.0
TC_IMAGE_HALVES = 3 * 4096          # per round: 2**11 Uh, Ul (one 128-row operand), Uh (FP16 bits)

# half index of B[n][k] in the K-major FP16 core-matrix layout (LBO 128 B, SBO 1024 B)
_N, _K = np.meshgrid(np.arange(64), np.arange(64), indexing='ij')
_KMAJOR = ((_N % 8) * 8 + (_K % 8) + (_K // 8) * 64 + (_N // 8) * 512).reshape(-1)


def tc_round_image(U):
    """12288 uint16 (FP16 bits) of U (64x64, FP64), each K-major: 2**11 Uh, Ul = fp16(2**11 (U - Uh)), Uh.

    The first two images are adjacent so that they form one 128-row operand."""
    U = np.asarray(U, dtype=np.float64)
    uh = U.astype(np.float16)
    parts = [(uh.astype(np.float64) * TC_LO_SCALE).astype(np.float16),
             ((U - uh.astype(np.float64)) * TC_LO_SCALE).astype(np.float16), uh]
    img = np.zeros(TC_IMAGE_HALVES, dtype=np.uint16)
    for i, part in enumerate(parts):
        img[4096 * i + _KMAJOR] = part.view(np.uint16).reshape(-1)
    return img


def pad_pass(p, n, k=TC_AXES):
    """Grow a pass's resident set to exactly k axes (adding the lowest free qubits)."""
    axes = set(p.axes)
    q = n - 1
    while len(axes) < k and q >= 0:
        axes.add(q)
        q -= 1
    return Pass(sorted(axes, reverse=True), p.ops)


# ---------------------------------------------------------------------------
# tensor-core round layouts
#
# A tensor-core round views the 4**7-coefficient tile as a 256 x 64 FP16
# operand (rows: groups, K: the round's 64 coefficients) in the K-major
# core-matrix layout: byte(row, k) = (row%8)*16 + (k%8)*2 + (k/8)*128 +
# (row/8)*1024.  Which tile bits form the row index, and in which order the
# round's three axes form the K digits, is free: the host picks them so that
# the epilogue of each round (one row per thread) writes the next round's
# operand with 64-bit stores (four FP16 values along one axis) whose
# half-warp phases hit distinct banks.  Tile bit 2a / 2a+1 is the low / high
# bit of local axis a's digit.
# ---------------------------------------------------------------------------

TC_A_BYTES = 256 * 64 * 2           # one FP16 operand image (hi or lo)


def _row_off(row):
    return (row & 7) * 16 + (row >> 3) * 1024


def _k_off(k):
    return (k & 7) * 2 + (k >> 3) * 128


def nat_swz(e):
    """Shared-memory element position of tile element e in the natural (streamed) layout."""
    return e ^ ((((e >> 5) ^ (e >> 8)) & 7) << 2)


def nat_linear(e):
    """Element position of tile element e in a TMA box (dense, unswizzled)."""
    return e


# natural-tile layouts: 'xor' for the cp.async-fed pass (dm_apply_pass_tc), 'linear' for the TMA-fed pass
NAT_MAPS = {'xor': nat_swz, 'linear': nat_linear}


_ROW_BIT_BYTES = tuple(_row_off(1 << i) for i in range(8))   # operand byte offset of row bit i
_K_BIT_BYTES = tuple(_k_off(1 << i) for i in range(6))       # operand byte offset of K bit i


class TcLayout:
    """Digit order (3 local axes) and row-bit order (8 tile bits) of one round's operand."""

    __slots__ = ('digits', 'rowbits', 'kbits', '_byte')

    def __init__(self, digits, rowbits):
        self.digits = list(digits)
        self.rowbits = list(rowbits)
        self.kbits = [2 * a + b for a in self.digits for b in (0, 1)]
        byte = dict(zip(self.rowbits, _ROW_BIT_BYTES))
        byte.update(zip(self.kbits, _K_BIT_BYTES))
        self._byte = byte

    def byte_of_bit(self, tb):
        return self._byte[tb]


@functools.lru_cache(maxsize=None)
def _store_wavefronts(lane_offs, vec_bytes):
    """Shared-memory wavefronts of one warp store whose lane i writes at XOR of lane_offs[bits of i].

    A per-store constant offset (the non-lane part of the address) XORs
    every address alike and does not change the count, so a whole epilogue
    costs (stores per thread) x this.  Phases: 32 lanes for 2/4-byte stores,
    16 for 8-byte, 8 for 16-byte."""
    lanes = np.arange(32)
    addr = np.zeros(32, dtype=np.int64)
    for i, o in enumerate(lane_offs):
        addr ^= ((lanes >> i) & 1) * o
    phase = 32 if vec_bytes <= 4 else 128 // vec_bytes
    nw = max(1, vec_bytes // 4)
    total = 0
    for ph in range(32 // phase):
        words = np.unique((addr[ph * phase:(ph + 1) * phase, None] // 4 + np.arange(nw)[None, :]).reshape(-1))
        total += int(np.bincount(words % 32, minlength=32).max())
    return total


def _transition_cost(src, dst_off, vec):
    """Store wavefronts + issue of one warp's epilogue from layout src into byte offsets dst_off(tile bit)."""
    lane_offs = tuple(dst_off(tb) for tb in src.rowbits[:5])
    if vec:
        w, n = _store_wavefronts(lane_offs, vec), 16
    else:
        w, n = _store_wavefronts(lane_offs, 2 if vec is None else 4), 64
    return n * w + n // 4


def _conversion_cost(layout, nat='xor'):
    """Shared-memory load wavefronts of one warp converting the natural tile into round 0 (layout).

    A warp's lanes are (row bits 0-2, chunk bits = K bits 3-4) of 8-value
    chunks; with local axis 0 as digit 0 the 8 values are two 16-byte loads,
    otherwise eight 4-byte loads."""
    f = NAT_MAPS[nat]
    offs = tuple(4 * f(1 << tb) for tb in layout.rowbits[:3]) + \
        tuple(4 * f(1 << tb) for tb in layout.kbits[3:5])
    vec = layout.digits[0] == 0
    w = _store_wavefronts(offs, 16 if vec else 4)
    return (2 if vec else 8) * w


def _natural_cost(layout, nat='xor'):
    vec = 16 if _vec_digit(layout, 0) >= 0 else 0
    f = NAT_MAPS[nat]
    return _transition_cost(layout, lambda tb: 4 * f(1 << tb), vec)


def _fill_rows(first, lanes, keep, nonround):
    rowbits = list(first)
    for tb in lanes + keep + nonround:   # remaining lane bits, the previous order, new bits
        if tb not in rowbits:
            rowbits.append(tb)
    return rowbits


def _best_next_cost(cand, next_axes):
    """Cheapest epilogue from ``cand`` into a round on next_axes (lookahead of the greedy choice).

    It depends only on the candidate's row order and its set of axes (which
    decides whether the next round's digit 0 can take 8-byte stores)."""
    return _best_next_cost_cached(tuple(cand.rowbits), frozenset(cand.digits), tuple(sorted(next_axes)))


@functools.lru_cache(maxsize=65536)
def _best_next_cost_cached(rowbits, digit_set, next_axes):
    import itertools
    nonround = [tb for tb in range(2 * TC_AXES) if tb // 2 not in next_axes]
    lanes = [tb for tb in rowbits[:5] if tb in nonround]
    keep = [tb for tb in rowbits if tb in nonround]
    rows = _fill_rows(lanes[:3], lanes, keep, nonround)
    lane_bits = rowbits[:5]
    best = None
    for digits in itertools.permutations(next_axes):
        nxt = TcLayout(list(digits), rows)
        vec = 8 if nxt.digits[0] in digit_set else None
        lane_offs = tuple(nxt.byte_of_bit(tb) for tb in lane_bits)
        if vec:
            c = 16 * _store_wavefronts(lane_offs, vec) + 4
        else:
            c = 64 * _store_wavefronts(lane_offs, 2) + 16
        best = c if best is None or c < best else best
    return best


@functools.lru_cache(maxsize=4096)
def _choose_layouts_cached(rounds_axes, nat='xor', direct=False):
    import itertools
    layouts = []
    prev = None
    nlast = len(rounds_axes) - 1
    for ri, axes in enumerate(rounds_axes):
        axes = sorted(axes)
        nonround = [tb for tb in range(2 * TC_AXES) if tb // 2 not in axes]
        nxt_axes = set(rounds_axes[ri + 1]) if ri < nlast else None
        if direct and ri == nlast and prev is not None:
            # the last round stores to global memory: rows 0-3 on tile bits 0-3, chosen by the cost
            # of the epilogue into it
            best = None
            for d, rows in _tma_last_candidates(axes, prev):
                cand = TcLayout(list(d), rows)
                vec = 8 if _vec_digit(prev, cand.digits[0]) >= 0 else None
                cost = _transition_cost(prev, cand.byte_of_bit, vec)
                if best is None or cost < best[0]:
                    best = (cost, cand)
            layouts.append(best[1])
            break
        if prev is None:
            # round 0: its rows 0-2 and K bits 3-4 are the lanes of the conversion's natural-tile
            # loads; its rows 0-4 the lanes of its own epilogue
            orders = [[0] + [a for a in axes if a != 0]] if 0 in axes else list(itertools.permutations(axes))
            best = None
            for digits in orders:
                for tri in itertools.combinations(nonround, 3):
                    cand = TcLayout(list(digits), _fill_rows(list(tri), [], [], nonround))
                    cost = _conversion_cost(cand, nat)
                    cost += _best_next_cost(cand, nxt_axes) if nxt_axes else _natural_cost(cand, nat)
                    if best is None or cost < best[0]:
                        best = (cost, cand)
            layouts.append(best[1])
            prev = best[1]
            continue
        lanes = [tb for tb in prev.rowbits[:5] if tb in nonround]
        keep = [tb for tb in prev.rowbits if tb in nonround]
        triples = list(itertools.combinations(lanes, 3)) if len(lanes) >= 3 else [tuple(lanes)]
        # row 3 feeds the next epilogue's 16-lane phases: the low bit of an axis the next round
        # adds can become its K bit 2 (byte 8), which keeps those 8-byte stores conflict-free
        fourth = [None] + ([tb for tb in nonround if tb % 2 == 0 and tb // 2 in nxt_axes] if nxt_axes else [])
        best = None
        for digits in itertools.permutations(axes):
            for tri in triples:
                for f in fourth:
                    if f in tri:
                        continue
                    cand = TcLayout(list(digits), _fill_rows(list(tri) + ([f] if f is not None else []),
                                                             lanes, keep, nonround))
                    vec = 8 if _vec_digit(prev, cand.digits[0]) >= 0 else None
                    cost = _transition_cost(prev, cand.byte_of_bit, vec)
                    cost += _natural_cost(cand, nat) if ri == nlast else _best_next_cost(cand, nxt_axes)
                    if best is None or cost < best[0]:
                        best = (cost, cand)
        layouts.append(best[1])
        prev = best[1]
    return tuple(layouts)


# Layouts of the TMA-fed pass (dm_apply_pass_tma).  Its first round converts
# the natural tile with one thread per operand row and its last round stores
# one row per thread straight to global memory; both keep tile bits 0-3
# (local axes 0 and 1, the 16 contiguous coefficients of a tile) as row bits
# 0-3, so the 32 lanes of a warp read and write runs of 16 consecutive
# coefficients.
TMA_FIXED_ROWS = [0, 1, 2, 3]


def _tma_conversion_cost(layout):
    """Shared-memory load wavefronts of one warp converting the natural tile: 64 word loads, lanes = rows 0-4."""
    return 64 * _store_wavefronts(tuple(4 * (1 << tb) for tb in layout.rowbits[:5]), 4)


@functools.lru_cache(maxsize=4096)
def _choose_layouts_tma_cached(rounds_axes):
    import itertools
    nlast = len(rounds_axes) - 1
    layouts = []
    prev = None

    fixed_cache = {}
    into_last = {}

    def fixed_next(nxt_axes):
        """The layouts the next round may take when it is the last round (its rows are fixed)."""
        key = tuple(sorted(nxt_axes))
        if key not in fixed_cache:
            fixed_cache[key] = [TcLayout(list(d), r) for d, r in _tma_last_candidates(list(key), None)]
        return fixed_cache[key]

    for ri, axes in enumerate(rounds_axes):
        axes = sorted(axes)
        nonround = [tb for tb in range(2 * TC_AXES) if tb // 2 not in axes]
        nxt_axes = set(rounds_axes[ri + 1]) if ri < nlast else None
        cands = []
        if ri == nlast:
            cands = [TcLayout(list(d), r) for d, r in _tma_last_candidates(axes, prev)]
        elif ri == 0:
            if all(tb in nonround for tb in TMA_FIXED_ROWS):
                # rows 0-4 hold tile bits 0-3 and one more bit in any order: conflict-free word loads
                rest = [tb for tb in nonround if tb not in TMA_FIXED_ROWS]
                fifth = ([4] if 4 in rest else []) + [tb for tb in rest if tb != 4][:2]
                for digits in itertools.permutations(axes):
                    for f in fifth:
                        tail = [tb for tb in rest if tb != f]
                        for head in itertools.permutations(TMA_FIXED_ROWS + [f]):
                            cands.append(TcLayout(list(digits), list(head) + tail))
            else:            # round 0 acts on local axis 0 or 1: lanes on the lowest free tile bits
                low = nonround[:5]
                for digits in itertools.permutations(axes):
                    cands.append(TcLayout(list(digits), low + [tb for tb in nonround if tb not in low]))
        else:
            lanes = [tb for tb in prev.rowbits[:5] if tb in nonround]
            keep = [tb for tb in prev.rowbits if tb in nonround]
            triples = list(itertools.combinations(lanes, 3)) if len(lanes) >= 3 else [tuple(lanes)]
            fourth = [None] + ([tb for tb in nonround if tb % 2 == 0 and tb // 2 in nxt_axes] if nxt_axes else [])
            for digits in itertools.permutations(axes):
                for tri in triples:
                    for f in fourth:
                        if f in tri:
                            continue
                        cands.append(TcLayout(list(digits), _fill_rows(list(tri) + ([f] if f is not None else []),
                                                                       lanes, keep, nonround)))
        best = None
        for cand in cands:
            cost = _tma_conversion_cost(cand) if ri == 0 else 0
            if prev is not None:
                vec = 8 if _vec_digit(prev, cand.digits[0]) >= 0 else None
                cost += _transition_cost(prev, cand.byte_of_bit, vec)
            if ri < nlast:
                if ri + 1 == nlast:      # the last round's rows are fixed: its exact incoming cost
                    # (it depends only on the candidate's lane bits and its set of axes)
                    key = (tuple(cand.rowbits[:5]), frozenset(cand.digits), tuple(sorted(nxt_axes)))
                    if key not in into_last:
                        into_last[key] = min(
                            _transition_cost(cand, nxt.byte_of_bit, 8 if _vec_digit(cand, nxt.digits[0]) >= 0
                                             else None) for nxt in fixed_next(nxt_axes))
                    cost += into_last[key]
                else:
                    cost += _best_next_cost(cand, nxt_axes)
            if best is None or cost < best[0]:
                best = (cost, cand)
        layouts.append(best[1])
        prev = best[1]
    return tuple(layouts)


def _tma_last_candidates(axes, prev):
    """(digits, rowbits) candidates of the last round of a TMA-fed pass, which stores its rows to
    global memory: with local axis 0 among its axes, axis 0 is K digit 0 (four contiguous
    coefficients per thread, 16-byte stores); otherwise tile bits 0-3 (axes 0 and 1, or axis 0
    and the lowest free bits) are rows 0-3, so 16 lanes cover contiguous coefficients."""
    import itertools
    nonround = [tb for tb in range(2 * TC_AXES) if tb // 2 not in axes]
    out = []
    if 0 in axes:
        others = [a for a in axes if a != 0]
        rows = nonround
        for perm in itertools.permutations(others):
            out.append(([0] + list(perm), rows))
        return out
    head = [tb for tb in TMA_FIXED_ROWS if tb in nonround]
    head += [tb for tb in nonround if tb not in head][:4 - len(head)]
    rest = [tb for tb in nonround if tb not in head]
    for digits in itertools.permutations(axes):
        for h in itertools.permutations(head):      # rows 0-3 in any order: lanes 0-15 stay contiguous
            out.append((list(digits), list(h) + rest))
    return out


def direct_last_eligible(rounds_axes):
    """True when a cp.async-fed tensor-core pass can store its last round straight to global memory:
    at least two rounds, and the last one leaves local axes 0 and 1 alone (its rows 0-3 then hold
    tile bits 0-3, 16 contiguous coefficients per 16 lanes)."""
    return len(rounds_axes) >= 2 and not {0, 1} & set(rounds_axes[-1])


def _choose_layouts(rounds_axes, nat='xor', direct=False):
    """Pick each round's digit order and row-bit order (greedy along the rounds, one round of lookahead).

    The epilogue of round r (one source row per thread) writes round r+1's
    operand; its cost depends only on where the source's five lane bits land
    in the destination (bank bits 2-6: destination K bits 1-2 and row bits
    0-2) and on whether the destination's K digit 0 is one of the source's
    axes (8-byte vector stores).  Each candidate (digit order, which source
    lane bits become row bits 0-2, which bit becomes row 3) is scored by the
    exact wavefront count of its incoming epilogue plus the cheapest
    outgoing one; the last round pays for its stores into the natural tile
    (``nat`` names that tile's layout, see NAT_MAPS).
    """
    return list(_choose_layouts_cached(tuple(tuple(sorted(a)) for a in rounds_axes), nat, bool(direct)))


def _vec_digit(src, dst_first_axis):
    """Digit of ``src`` holding the destination's 4-vector axis, or -1."""
    return src.digits.index(dst_first_axis) if dst_first_axis in src.digits else -1


def epilogue_wavefronts(src, dst, natural=False):
    """Shared-memory store wavefronts of one warp writing src's rows 0..31 into dst's layout."""
    lanes = np.arange(32)

    def addr_bytes(row, k):
        e = 0
        for i, tb in enumerate(src.rowbits):
            if (row >> i) & 1:
                e |= 1 << tb
        for i, tb in enumerate(src.kbits):
            if (k >> i) & 1:
                e |= 1 << tb
        if natural:
            return 4 * nat_swz(e)
        return sum(dst.byte_of_bit(tb) for tb in range(2 * TC_AXES) if (e >> tb) & 1)

    vec_axis = 0 if natural else dst.digits[0]
    d = _vec_digit(src, vec_axis)
    vec_bytes = 16 if natural else 8     # four FP32 natural values / four FP16 operand values
    phase = 8 if natural else 16          # threads per shared-memory wavefront of that width
    total = 0
    if d >= 0:
        others = [j for j in range(64) if (j >> (2 * d)) & 3 == 0]
        for j in others:
            addrs = [addr_bytes(int(r), j) for r in lanes]
            for ph in range(32 // phase):
                cnt = {}
                for a in addrs[phase * ph:phase * ph + phase]:
                    for w in range(a // 4, (a + vec_bytes) // 4):
                        cnt.setdefault(w % 32, set()).add(w)
                total += max(len(v) for v in cnt.values())
    else:
        for j in range(64):
            words = [addr_bytes(int(r), j) // 4 for r in lanes]
            cnt = {}
            for w in words:
                cnt.setdefault(w % 32, set()).add(w)
            total += max(len(v) for v in cnt.values())
    return total


def plan_tc_rounds(p, n, nat='xor'):
    """Pad a pass to 7 axes, plan its rounds and their layouts: (pass, [(axes, ops)], layouts).

    nat='tma' plans for the TMA-fed kernel (first and last rounds with local
    axes 0 and 1 on rows 0-3 where they are not among the round's axes)."""
    pp = pad_pass(p, n)
    rounds = plan_rounds(pp, 3, pad='neighbors')
    if nat == 'tma':
        layouts = list(_choose_layouts_tma_cached(tuple(tuple(sorted(a)) for a, _ in rounds)))
    else:
        axes = [a for a, _ in rounds]
        layouts = _choose_layouts(axes, nat, direct=nat == 'xor' and direct_last_eligible(axes))
    return pp, rounds, layouts


def compose_round_matrices(rounds, layouts):
    """Each round's 64x64 U in its layout's digit order, composed in FP64 with numpy.

    The host statement of what dm_compose_rounds computes on the device."""
    mats = []
    for (axes, rops), lay in zip(rounds, layouts):
        U = np.eye(64)
        for op in rops:
            U = op_matrix64(op, lay.digits) @ U
        mats.append(U)
    return mats


def plan_tc_pass(p, n, nat='xor'):
    """plan_tc_rounds with each round's U composed on the host: (pass, layouts, [U])."""
    pp, rounds, layouts = plan_tc_rounds(p, n, nat)
    return pp, layouts, compose_round_matrices(rounds, layouts)


_ROUND_OP_KINDS = {'map1': (1, 16), 'cx': (4, 5), 'diag2': (3, 16), 'map2': (2, 256)}


def fill_round_ops(bp, pp, rounds, digit_orders, place):
    """Pass header, round axes (in ``digit_orders``) and ops of a DmBatchPass.

    ``place(op, flags, size)`` returns the op's coefficient offset (moff)
    after recording or storing its ``size`` coefficients.  The digit
    position of each op axis within its round goes into the flags (bits 8
    and 12), as the register rounds and the device composition read them."""
    bp.k = len(pp.axes)
    for r, q in enumerate(pp.axes):
        bp.axes[r] = q
    if len(rounds) > N.DM_MAX_ROUNDS:
        raise TcPlanError('pass needs %d rounds (> %d)' % (len(rounds), N.DM_MAX_ROUNDS))
    if sum(len(rops) for _, rops in rounds) > N.DM_MAX_PASS_OPS:
        raise OpTableError('pass holds more than %d ops' % N.DM_MAX_PASS_OPS)
    bp.nrounds = len(rounds)
    o = 0
    for ri, ((_, rops), axes) in enumerate(zip(rounds, digit_orders)):
        axes = list(axes)
        for i, a in enumerate(axes):
            bp.round_axes[ri][i] = a
        for i in range(len(axes), 4):
            bp.round_axes[ri][i] = -1
        for op in rops:
            if op.kind not in _ROUND_OP_KINDS:
                raise ValueError(op.kind)
            kind, size = _ROUND_OP_KINDS[op.kind]
            d = bp.ops[o]
            d.kind = kind
            d.a = op.axes[0]
            flags = axes.index(op.axes[0]) << 8
            if op.kind == 'map1':
                d.b = 0
                m = np.asarray(op.data).reshape(16)
                flags |= N.DM_MAP1_ROW0_IDENTITY if (m[0] == 1.0 and not m[1:4].any()) else 0
                flags |= N.DM_MAP1_XY_UNITAL if (m[4] == 0.0 and m[8] == 0.0) else 0
            else:
                d.b = op.axes[1]
                flags |= axes.index(op.axes[1]) << 12
                if op.kind == 'cx' and op.ideal:
                    flags |= N.DM_CX_IDEAL
            d.flags = flags
            d.moff = place(op, flags, size)
            o += 1
        bp.round_end[ri] = o
    bp.nops = o


def round_op_coefficients(op):
    """The FP64 coefficients of one op as a dm_op reads them (16, 5, 16 or 256 values)."""
    return np.ascontiguousarray(op.data, dtype=np.float64).reshape(-1)


def tc_tables(layouts, nat='xor', direct=False):
    """Conversion and per-round epilogue tables of a tensor-core pass (see dm_tc_pass); with
    ``direct`` the last round's are the linear natural offsets of its bits (global stores)."""
    f = NAT_MAPS[nat]
    L0 = layouts[0]
    conv = {'natrow': [f(1 << tb) for tb in L0.rowbits], 'natk': [f(1 << tb) for tb in L0.kbits],
            'vec0': 0 if L0.digits[0] == 0 else -1}
    rounds = []
    for r, L in enumerate(layouts):
        if r + 1 < len(layouts):
            nxt = layouts[r + 1]
            rowc = [nxt.byte_of_bit(tb) for tb in L.rowbits]
            kc = [nxt.byte_of_bit(tb) for tb in L.kbits]
            vec = _vec_digit(L, nxt.digits[0])
        elif direct:
            rowc = [1 << tb for tb in L.rowbits]
            kc = [1 << tb for tb in L.kbits]
            vec = -1
        else:
            rowc = [f(1 << tb) for tb in L.rowbits]
            kc = [f(1 << tb) for tb in L.kbits]
            vec = _vec_digit(L, 0)
        rounds.append({'digits': L.digits, 'rowc': rowc, 'kc': kc, 'vec': vec})
    return conv, rounds


def _encode_tc(pp, layouts, nat, umoff0, halves):
    """DmTcPass tables of a planned pass; round r reads its image at umoff0 + r * halves."""
    if len(layouts) > N.DM_MAX_ROUNDS:
        raise TcPlanError('pass needs %d rounds (> %d)' % (len(layouts), N.DM_MAX_ROUNDS))
    direct = nat == 'xor' and direct_last_eligible([L.digits for L in layouts])
    conv, rounds = tc_tables(layouts, nat, direct)
    dp = N.DmTcPass()
    dp.direct_last = 1 if direct else 0
    for r, q in enumerate(pp.axes):
        dp.axes[r] = q
    dp.nrounds = len(layouts)
    dp.vec0 = conv['vec0']
    for i in range(8):
        dp.natrow[i] = conv['natrow'][i]
    for i in range(6):
        dp.natk[i] = conv['natk'][i]
    for ri, rd in enumerate(rounds):
        o = dp.rounds[ri]
        for i in range(3):
            o.digits[i] = rd['digits'][i]
        o.vec = rd['vec']
        for i in range(8):
            o.rowc[i] = rd['rowc'][i]
        for i in range(6):
            o.kc[i] = rd['kc'][i]
        o.umoff = umoff0 + ri * halves
    return dp


def encode_pass_tc(p, n, umats):
    """DmTcPass for dm_apply_pass_tc; appends the rounds' FP16 matrix images (uint16) to ``umats``."""
    pp, layouts, mats = plan_tc_pass(p, n)
    dp = _encode_tc(pp, layouts, 'xor', sum(m.size for m in umats), TC_IMAGE_HALVES)
    umats.extend(tc_round_image(U) for U in mats)
    return dp


def encode_pass_tc_ops(p, n, coefs, kernel='tc'):
    """(DmTcPass, DmBatchPass) of a tensor-core pass whose round images the device composes.

    kernel 'tc' (dm_apply_pass_tc, images of TC_IMAGE_HALVES) or 'tma'
    (dm_apply_pass_tma, TMA_IMAGE_HALVES).  The DmTcPass reads round r's
    image at r * (image values): dm_compose_rounds writes them there from the
    DmBatchPass's ops, whose FP64 coefficients are appended to ``coefs``
    (a list of arrays; moff counts from its start).  Raises TcPlanError for
    a pass that does not fit the kernel or the op table."""
    nat = 'tma' if kernel == 'tma' else 'xor'
    pp, rounds, layouts = plan_tc_rounds(p, n, nat)
    if kernel == 'tma' and not tma_eligible(pp, n, layouts):
        raise TcPlanError('pass does not fit the TMA-fed kernel (%d rounds, dims %s)'
                          % (len(layouts), tma_box_dims(n, pp.axes)))
    halves = TMA_IMAGE_HALVES if kernel == 'tma' else TC_IMAGE_HALVES
    bp = N.DmBatchPass()
    off = [sum(c.size for c in coefs)]

    def place(op, flags, size):
        c = round_op_coefficients(op)
        assert c.size == size
        coefs.append(c)
        off[0] += size
        return off[0] - size

    dp = _encode_tc(pp, layouts, 'linear' if kernel == 'tma' else 'xor', 0, halves)
    fill_round_ops(bp, pp, rounds, [L.digits for L in layouts], place)
    return dp, bp


# ---------------------------------------------------------------------------
# TMA-fed tensor-core pass (dm_apply_pass_tma)
# ---------------------------------------------------------------------------

TMA_MAX_ROUNDS = 16       # rounds of one pass (up to 6 with every round image resident, more streamed)
TMA_MAX_DIMS = 5          # tensor-map rank
TMA_IMAGE_HALVES = 2 * 4096


def tc_round_image_tma(U):
    """8192 uint16 (FP16 bits) of U (64x64, FP64), each K-major: Uh, then Ul = fp16(2**11 (U - Uh)).

    Adjacent, so that [Uh ; Ul] is one 128-row operand (h x [Uh ; Ul]) and
    its first half the operand of l x Uh."""
    U = np.asarray(U, dtype=np.float64)
    uh = U.astype(np.float16)
    parts = [uh, ((U - uh.astype(np.float64)) * TC_LO_SCALE).astype(np.float16)]
    img = np.zeros(TMA_IMAGE_HALVES, dtype=np.uint16)
    for i, part in enumerate(parts):
        img[4096 * i + _KMAJOR] = part.view(np.uint16).reshape(-1)
    return img


def tma_box_dims(n, axes):
    """Tensor-map dimensions of a tile of resident qubits ``axes``: [(start digit, length, gap above)].

    Runs of consecutive resident digit positions (qubit q has position
    n-1-q), split into chunks of at most 4 digits; gap counts the
    non-resident digits between a chunk and the next one (or the top).
    Mirrors tma_dims() in csrc/dm_tma.cu."""
    res = set(n - 1 - q for q in axes)
    dims, pos = [], 0
    if 0 not in res:
        return None
    while pos < n:
        length = 0
        while pos + length < n and pos + length in res and length < 4:
            length += 1
        gap = 0
        while pos + length + gap < n and pos + length + gap not in res:
            gap += 1
        dims.append((pos, length, gap))
        pos += length + gap
    return dims


def tma_eligible(pp, n, layouts):
    """True when dm_apply_pass_tma takes the pass planned as ``layouts`` (plan_tc_pass(..., nat='tma')).

    Not when the last round acts on both local axes 0 and 1: its rows then hold
    none of the tile's contiguous coefficients, so every lane's stores land in
    a different place (measured: about three times the pass's time on
    pass_tc_kernel)."""
    dims = tma_box_dims(n, pp.axes)
    return layouts is not None and dims is not None and len(dims) <= TMA_MAX_DIMS \
        and len(layouts) <= TMA_MAX_ROUNDS and not {0, 1} <= set(layouts[-1].digits)


def encode_pass_tma(p, n, umats):
    """DmTcPass for dm_apply_pass_tma: natural-tile tables as plain element offsets (the TMA box is
    unswizzled; the last round's are turned into global offsets by the library), [Uh ; Ul] images.

    Raises TcPlanError when the pass has more than TMA_MAX_ROUNDS rounds or
    its resident digits need more tensor-map dimensions than TMA has."""
    pp, layouts, mats = plan_tc_pass(p, n, nat='tma')
    if not tma_eligible(pp, n, layouts):
        raise TcPlanError('pass does not fit the TMA-fed kernel (%d rounds, dims %s)'
                          % (len(layouts), tma_box_dims(n, pp.axes)))
    dp = _encode_tc(pp, layouts, 'linear', sum(m.size for m in umats), TMA_IMAGE_HALVES)
    umats.extend(tc_round_image_tma(U) for U in mats)
    return dp
