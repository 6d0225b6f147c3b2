"""Host-side scheduling with the reference's semantics: single-qubit gate
merging and levelling into clock cycles.

The number of levels matters for the physics, not only for speed: the
reference applies memory noise to every qubit once per level
(dm_simulator.py:1173-1177), so the GPU engine must reproduce the
reference's levels exactly.

* ``merge_single_gates``  -- basicaertools.py:251-307 (single_gate_merge),
  with the pair merge of :181-228 (mergeU) and the Euler-angle conversion
  of :129-178 (U3_merge).
* ``levelize``            -- basicaertools.py:714-749 (partition), built on
  :536-591 (qubit_stack) and :594-712 (partition_helper); the levelling itself
  runs in the library (dm_levelize, csrc/dm_sched.cpp).

Both keep the reference's observable behaviour: merged instructions are
emitted at each separator in qubit order, a merged run keeps the position
of its earliest gate, measurements and resets get their own levels (with
"dummy" placeholders on the other qubits), and the level list is the
concatenation of each barrier-separated piece's pre-sized level table
(including unused trailing entries), of which the first ``levels`` entries
are executed.
"""
import copy
import math

import numpy as np

from .exceptions import QiskitError

_SEPARATORS = frozenset(('CX', 'cx', 'measure', 'bfunc', 'reset', 'barrier'))
_ROTATIONS = frozenset(('U', 'u1', 'u2', 'u3'))


def euler_zyz_from_yzy(xi, th1, th2):
    """Ry(th1) Rz(xi) Ry(th2) rewritten as Rz(alpha) Ry(beta) Rz(gamma): (beta, alpha, gamma)."""
    s_xi, c_xi = math.sin(xi / 2), math.cos(xi / 2)
    a, b = (th1 + th2) / 2, (th1 - th2) / 2
    s_a, c_a, s_b, c_b = math.sin(a), math.cos(a), math.sin(b), math.cos(b)
    p = math.atan2(s_xi * c_b, c_xi * c_a)       # (alpha + gamma) / 2
    m = math.atan2(-s_xi * s_b, c_xi * s_a)      # (alpha - gamma) / 2
    beta = 2 * math.acos(math.sqrt((c_xi * c_a) ** 2 + (s_xi * c_b) ** 2))
    return beta, p + m, p - m


def _combine(older, newer):
    """Combine two rotations on one qubit; ``older`` acts first.

    Each argument is (instruction, position).  The result is a copy of the
    earlier-positioned instruction carrying the combined parameters.
    """
    (g1, i1), (g2, i2) = older, newer
    out = copy.deepcopy(older if i1 < i2 else newer)
    op = out[0]
    n1, n2 = g1.name, g2.name
    if n1 == 'u1' and n2 == 'u1':
        op.params[0] = g1.params[0] + g2.params[0]
    elif n1 == 'u1' or n2 == 'u1':
        if op.name == 'u1':
            op.name = 'u3'
            op.params += [0, 0]
        if n1 == 'u1':           # u1 then u3: lambda absorbs the u1 angle
            op.params[0], op.params[1], op.params[2] = g2.params[0], g2.params[1], g2.params[2] + g1.params[0]
        else:                    # u3 then u1: phi absorbs the u1 angle
            op.params[0], op.params[1], op.params[2] = g1.params[0], g1.params[1] + g2.params[0], g1.params[2]
    elif n1 == 'u3' and n2 == 'u3':
        beta, alpha, gamma = euler_zyz_from_yzy(float(g2.params[2] + g1.params[1]),
                                                float(g2.params[0]), float(g1.params[0]))
        op.params[0] = beta
        op.params[1] = g2.params[1] + alpha
        op.params[2] = g1.params[2] + gamma
    else:
        raise QiskitError('Encountered unrecognized instructions: %s, %s' % (n1, n2))
    return out


def _fold(run):
    if len(run) == 1:
        return run[0][0]
    acc = run[0]
    for nxt in run[1:]:
        acc = _combine(acc, nxt)
    return acc[0]


def _canonical_name(op):
    if op.name == 'CX':
        op.name = 'cx'
    elif op.name == 'U':
        op.name = 'u3'
    elif op.name == 'u2':
        op.name = 'u3'
        op.params.insert(0, np.pi / 2)


def merge_single_gates(insts, n, merge=True):
    """Merge runs of single-qubit rotations between separators (mutates names/params)."""
    if not merge:
        out = []
        for op in insts:
            _canonical_name(op)
            if op.name not in ('id', 'u0'):
                out.append(op)
        return out
    runs = {}
    out = []
    for pos, op in enumerate(insts):
        name = op.name
        if name in _SEPARATORS:
            for q in sorted(runs):
                out.append(_fold(runs[q]))
            runs.clear()
            _canonical_name(op)
            out.append(op)
        elif name in _ROTATIONS:
            _canonical_name(op)
            runs.setdefault(op.qubits[0], []).append((op, pos))
        elif name in ('id', 'u0'):
            continue
        else:
            raise QiskitError('Encountered unrecognized instruction: %s' % name)
    for q in sorted(runs):
        out.append(_fold(runs[q]))
    return out


# ---------------------------------------------------------------------------
# levelling (compiled: dm_levelize in csrc/dm_sched.cpp)
# ---------------------------------------------------------------------------

_KINDS = {'u1': 1, 'u3': 1, 'cx': 2, 'CX': 2, 'measure': 3, 'reset': 4, 'barrier': 5}


def levelize(insts, n):
    """Split on barriers and level each piece; returns (level table, number of levels).

    The levels are computed by the library's dm_levelize (the reference's
    partition, basicaertools.py:536-749, in C++); the table lists the
    instruction objects of each level in the order the reference appends them.
    """
    import ctypes
    from . import _native as N
    count = len(insts)
    kind = np.empty(count, dtype=np.int32)
    qoff = np.zeros(count + 1, dtype=np.int32)
    qubits = []
    for i, op in enumerate(insts):
        kind[i] = _KINDS.get(op.name, N.DM_SCHED_OTHER)
        qs = [] if op.name == 'barrier' else [int(q) for q in op.qubits]
        qubits.extend(qs)
        qoff[i + 1] = qoff[i] + len(qs)
    qarr = np.asarray(qubits if qubits else [0], dtype=np.int32)
    placed_inst = np.empty(max(count, 1), dtype=np.int32)
    placed_pos = np.empty(max(count, 1), dtype=np.int32)
    out = np.zeros(3, dtype=np.int32)

    def ptr(a, k=0):
        return ctypes.c_void_p(a.ctypes.data + 4 * k)

    rc = N.lib().dm_levelize(n, count, ptr(kind), ptr(qoff), ptr(qarr), ptr(placed_inst), ptr(placed_pos),
                             ptr(out, 0), ptr(out, 1), ptr(out, 2))
    if rc == N.DM_ERR_PROGRAM:
        raise QiskitError('levelling cannot place the remaining instructions')
    if rc != N.DM_OK:
        raise QiskitError('levelling failed: %s' % N.lib().dm_error_string(rc).decode())
    placed, table_len, levels = (int(x) for x in out)
    table = [[] for _ in range(table_len)]
    for k in range(placed):
        table[placed_pos[k]].append(insts[placed_inst[k]])
    return table, levels
