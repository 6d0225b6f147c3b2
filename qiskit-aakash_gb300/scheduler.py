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
  :536-591 (qubit_stack) and :594-712 (partition_helper).

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
# levelling
# ---------------------------------------------------------------------------

class _Placeholder:
    """Stands on a qubit's stack for a measurement / reset on another qubit."""
    __slots__ = ('kind',)

    def __init__(self, kind):
        self.kind = kind


def _stacks(piece, n):
    stacks = [[] for _ in range(n)]
    for op in piece:
        kind = op.name
        if kind not in ('measure', 'reset'):
            for q in op.qubits:
                stacks[q].append(op)
            continue
        q0 = op.qubits[0]
        top = stacks[q0][-1] if stacks[q0] else None
        if isinstance(top, _Placeholder) and top.kind == kind:
            stacks[q0][-1] = op           # joins the pending simultaneous group
            continue
        stacks[q0].append(op)
        ph = _Placeholder(kind)
        for q in range(n):
            if q not in op.qubits:
                stacks[q].append(ph)
    return stacks


def _level_piece(piece, n):
    stacks = _stacks(piece, n)
    heads = [0] * n
    table = [[] for _ in range(max(len(s) for s in stacks))]
    remaining = len(piece)
    level = 0

    def top(q):
        return stacks[q][heads[q]] if heads[q] < len(stacks[q]) else None

    while remaining:
        busy = set()
        placed_before = remaining
        if level == len(table):
            table.append([])
        for q in range(n):
            g = top(q)
            if g is None or isinstance(g, _Placeholder):
                continue
            name = g.name
            if name in ('u3', 'u1'):
                if q in busy:
                    continue
                table[level].append(g)
                busy.add(q)
                heads[q] += 1
                remaining -= 1
            elif name in ('cx', 'CX'):
                other = [x for x in g.qubits if x != q][0]
                partner = top(other)
                if q in busy or other in busy or partner is not g:
                    continue
                busy.update((q, other))
                table[level].append(g)
                heads[q] += 1
                heads[other] += 1
                remaining -= 1
            elif name in ('measure', 'reset'):
                ready = all(t is None or (isinstance(t, _Placeholder) and t.kind == name)
                            or (not isinstance(t, _Placeholder) and t.name == name)
                            for t in (top(x) for x in range(n)))
                if not ready:
                    if not remaining:
                        break
                    continue
                if table[level]:
                    busy = set()
                    level += 1
                    if level == len(table):
                        table.append([])
                for x in range(n):
                    t = top(x)
                    if t is None:
                        continue
                    if not isinstance(t, _Placeholder):
                        busy.add(x)
                        table[level].append(t)
                        remaining -= 1
                    heads[x] += 1
                break
            if not remaining:
                break
        if remaining == placed_before:
            raise QiskitError('levelling cannot place the remaining instructions')
        level += 1
    return table, level


def levelize(insts, n):
    """Split on barriers and level each piece; returns (level table, number of levels)."""
    pieces, cur = [], []
    for op in insts:
        if op.name == 'barrier':
            pieces.append(cur)
            cur = []
        else:
            cur.append(op)
    if cur:
        pieces.append(cur)
    table, levels = [], 0
    for piece in pieces:
        if not piece:
            continue
        head = piece[0]
        prm = getattr(head, 'params', None)
        if head.name == 'measure' and prm and isinstance(prm[0], str) \
                and prm[0] in ('Bell', 'Expect', 'Ensemble'):
            # Plain-string parameters (never produced by qiskit's assembler,
            # which makes them sympy Symbols) send the reference down a path
            # that fails (basicaertools.py:740-747); level them like Symbols.
            pass
        t, lv = _level_piece(piece, n)
        table.extend(t)
        levels += lv
    return table, levels
