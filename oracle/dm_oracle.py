"""CPU oracle for the Pauli-basis density-matrix path (TEST INFRASTRUCTURE ONLY).

This module restates, in numpy FP64 on the host, the algorithm of the
reference backend ``dm_simulator`` (qiskit-aakash):

* ``qiskit/providers/basicaer/basicaertools.py``  -- rotation / CX kernels,
  single-qubit gate merging and the levelling ("partition") pass;
* ``qiskit/providers/basicaer/dm_simulator.py``   -- options, initial states,
  memory noise, the measurement family and the level loop.

Every function cites the reference lines it follows.  The state is the real
vector of 4**n Pauli coefficients with flat index sum_q p_q * 4**(n-1-q),
p in {0:I, 1:X, 2:Y, 3:Z}: qubit 0 is the slowest axis.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this module, as the checker / the timed CPU baseline.  The
GB300 product path never calls it.

Parity of this restatement is pinned against the reference itself: the
fixtures under ``tests/golden/`` were produced by running the unmodified
reference files (``tests/golden/make_golden.py``) and ``tests/test_oracle.py``
checks this module against them.
"""
import copy
import itertools
import logging
import math

import numpy as np

logger = logging.getLogger(__name__)


class OracleError(Exception):
    """Stands in for the reference's BasicAerError / QiskitError."""


# ---------------------------------------------------------------------------
# single-qubit gate merging  (basicaertools.py:129-307)
# ---------------------------------------------------------------------------

def u3_merge_angles(xi, th1, th2):
    """Ry(th1) Rz(xi) Ry(th2) -> (beta, alpha, gamma) of Rz(alpha) Ry(beta) Rz(gamma).

    basicaertools.py:129-178 (U3_merge).
    """
    sx, cx = math.sin(0.5 * xi), math.cos(0.5 * xi)
    sp, cp = math.sin(0.5 * (th1 + th2)), math.cos(0.5 * (th1 + th2))
    sm, cm = math.sin(0.5 * (th1 - th2)), math.cos(0.5 * (th1 - th2))
    half_sum = math.atan2(sx * cm, cx * cp)
    half_diff = math.atan2(-sx * sm, cx * sp)
    beta = 2.0 * math.acos(math.sqrt((cx * cp) ** 2 + (sx * cm) ** 2))
    return beta, half_sum + half_diff, half_sum - half_diff


def merge_pair(first, second):
    """Merge two [instruction, index] entries on one qubit.  basicaertools.py:181-228."""
    keep = copy.deepcopy(first if first[1] < second[1] else second)
    a, b = first[0], second[0]
    if a.name == 'u1' and b.name == 'u1':
        keep[0].params[0] = a.params[0] + b.params[0]
    elif a.name == 'u1' or b.name == 'u1':
        if keep[0].name == 'u1':
            keep[0].name = 'u3'
            keep[0].params.extend([0, 0])
        if a.name == 'u1' and b.name == 'u3':
            keep[0].params[0:3] = [b.params[0], b.params[1], b.params[2] + a.params[0]]
        elif a.name == 'u3' and b.name == 'u1':
            keep[0].params[0:3] = [a.params[0], a.params[1] + b.params[0], a.params[2]]
    elif a.name == 'u3' and b.name == 'u3':
        beta, alpha, gamma = u3_merge_angles(float(b.params[2] + a.params[1]),
                                             float(b.params[0]), float(a.params[0]))
        keep[0].params[0] = beta
        keep[0].params[1] = b.params[1] + alpha
        keep[0].params[2] = a.params[2] + gamma
    else:
        raise OracleError('Encountered unrecognized instructions: %s, %s' % (a.name, b.name))
    return keep


def merge_run(run):
    """basicaertools.py:231-248 (merge_gates)."""
    if len(run) < 2:
        return run[0][0]
    acc = merge_pair(run[0], run[1])
    for entry in run[2:]:
        acc = merge_pair(acc, entry)
    return acc[0]


_SEPARATORS = ('CX', 'cx', 'measure', 'bfunc', 'reset', 'barrier')


def merge_single_gates(insts, n, merge=True):
    """basicaertools.py:251-307 (single_gate_merge).  Mutates names/params like the reference."""
    out = []
    if not merge:
        for op in insts:
            if op.name == 'CX':
                op.name = 'cx'
            elif op.name == 'U':
                op.name = 'u3'
            elif op.name == 'u2':
                op.name = 'u3'
                op.params.insert(0, np.pi / 2)
            if op.name not in ('id', 'u0'):
                out.append(op)
        return out
    pending = [[] for _ in range(n)]
    for idx, op in enumerate(insts):
        if op.name in _SEPARATORS:
            for q in range(n):
                if pending[q]:
                    out.append(merge_run(pending[q]))
                    pending[q] = []
            if op.name == 'CX':
                op.name = 'cx'
            out.append(op)
        elif op.name in ('U', 'u1', 'u2', 'u3'):
            if op.name == 'U':
                op.name = 'u3'
            elif op.name == 'u2':
                op.name = 'u3'
                op.params.insert(0, np.pi / 2)
            pending[op.qubits[0]].append([op, idx])
        elif op.name in ('id', 'u0'):
            continue
        else:
            raise OracleError('Encountered unrecognized instruction: %s' % op.name)
    for q in range(n):
        if pending[q]:
            out.append(merge_run(pending[q]))
    return out


# ---------------------------------------------------------------------------
# levelling  (basicaertools.py:536-749)
# ---------------------------------------------------------------------------

def _dummy_of(op, kind):
    d = copy.deepcopy(op)
    d.name = kind
    d.qubits[0] = -1
    return d


def per_qubit_stacks(insts, n):
    """basicaertools.py:536-591 (qubit_stack)."""
    stacks = [[] for _ in range(n)]
    for op in insts:
        if op.name not in ('measure', 'reset'):
            for q in op.qubits:
                stacks[q].append(op)
            continue
        dummy_name = 'dummy_' + op.name
        q0 = op.qubits[0]
        if stacks[q0] and stacks[q0][-1].name == dummy_name:
            stacks[q0][-1] = op
            continue
        stacks[q0].append(op)
        d = _dummy_of(op, dummy_name)
        for q in set(range(n)).difference(set(op.qubits)):
            stacks[q].append(d)
    return stacks, max(len(s) for s in stacks)


def _remove_identity(lst, item):
    # list.remove() compares with ==; qobj instructions compare by identity.
    for i, x in enumerate(lst):
        if x is item or x == item:
            del lst[i]
            return
    raise ValueError('item not in list')


def level_segment(insts, n):
    """basicaertools.py:594-712 (partition_helper)."""
    stacks, depth = per_qubit_stacks(insts, n)
    pool = list(insts)
    level, seq = 0, [[] for _ in range(depth)]
    while pool:
        taken = []
        before = len(pool)
        if level == len(seq):
            seq.append([])
        for q in range(n):
            if not stacks[q]:
                continue
            gate = stacks[q][0]
            if gate.name in ('dummy_measure', 'dummy_reset'):
                continue
            if gate.name in ('u3', 'u1'):
                if q in taken:
                    continue
                seq[level].append(gate)
                taken.append(q)
                _remove_identity(pool, gate)
                stacks[q].pop(0)
            elif gate.name in ('CX', 'cx'):
                other = list(set(gate.qubits).difference({q}))[0]
                partner_top = stacks[other][0]
                if q in taken or other in taken:
                    continue
                if gate is partner_top:
                    taken += [q, other]
                    seq[level].append(gate)
                    _remove_identity(pool, gate)
                    stacks[q].pop(0)
                    stacks[other].pop(0)
            elif gate.name in ('measure', 'reset'):
                kind = gate.name
                ready = True
                for x in range(n):
                    if stacks[x] and stacks[x][0].name not in (kind, 'dummy_' + kind):
                        ready = False
                        break
                if ready:
                    if seq[level]:
                        taken = []
                        level += 1
                        if level == len(seq):
                            seq.append([])
                    for x in range(n):
                        if not stacks[x]:
                            continue
                        if stacks[x][0].name == kind:
                            taken.append(x)
                            seq[level].append(stacks[x][0])
                            _remove_identity(pool, stacks[x][0])
                        stacks[x].pop(0)
                    break
            if not pool:
                break
        if len(pool) == before:
            # Nothing could be placed: the reference's while-loop never ends here.
            raise OracleError('levelling makes no progress (the reference loops forever)')
        level += 1
    return seq, level


def partition_levels(insts, n):
    """basicaertools.py:714-749 (partition): split on barriers, level each piece, chain."""
    pieces, cur = [], []
    for op in insts:
        if op.name != 'barrier':
            cur.append(op)
        else:
            pieces.append(cur)
            cur = []
    if cur:
        pieces.append(cur)
    chained, levels = [], 0
    for piece in pieces:
        if not piece:
            continue
        head = piece[0]
        # With qobj params (sympy Symbols) this test is False in the reference,
        # so Ensemble/Expect/Bell pieces are levelled like any other piece.
        if head.name == 'measure' and getattr(head, 'params', None) is not None \
                and any(head.params[0] is s or (isinstance(head.params[0], str) and head.params[0] == s)
                        for s in ('Bell', 'Expect', 'Ensemble')):
            # The reference chains this piece's bare instructions into the
            # level list and then fails iterating one of them.
            raise OracleError('string measurement parameters are not levelled by the reference')
        else:
            seq, lv = level_segment(piece, n)
            chained.extend(seq)
            levels += lv
    return chained, levels


# ---------------------------------------------------------------------------
# numpy kernels  (basicaertools.py:93-126, :310-392; dm_simulator.py:397-823)
# ---------------------------------------------------------------------------

_ROT_AXES = {'rz': (1, 2), 'ry': (3, 1), 'rx': (2, 3)}


def rotate(view, name, angle, err):
    """basicaertools.py:93-126 (rot_gate_dm_matrix) on a (4**q, 4, rest) view."""
    c = err[0] * np.cos(angle + err[1])
    s = err[0] * np.sin(angle + err[1])
    if name not in _ROT_AXES:
        raise OracleError('Gate is not among the valid decomposition types: %s' % name)
    k0, k1 = _ROT_AXES[name]
    old = view.copy()
    view[:, k0, :] = c * old[:, k0, :] - s * old[:, k1, :]
    view[:, k1, :] = c * old[:, k1, :] + s * old[:, k0, :]
    return view


def u_decomposition(name, params):
    """basicaertools.py:69-90 (single_gate_dm_matrix)."""
    p = [float(x) for x in params]
    if name in ('U', 'u3'):
        return [('rz', p[2]), ('ry', p[0]), ('rz', p[1])]
    if name == 'u1':
        return [('rz', p[0])]
    raise OracleError('Gate is not among the valid types: %s' % name)


def cx_apply(state, n, ctl, tgt, tsp):
    """basicaertools.py:310-392 (cx_gate_dm_matrix)."""
    cav = tsp[0]
    c2av = 4 * cav - 3
    c = cav * np.cos(tsp[1])
    s = cav * np.sin(tsp[1])
    c2 = 0.5 * (1 + c2av * np.cos(2 * tsp[1]))
    s2 = 0.5 * (1 - c2av * np.cos(2 * tsp[1]))
    cs = c2av * np.sin(tsp[1]) * np.cos(tsp[1])
    if ctl == tgt or ctl >= n or tgt >= n:
        raise OracleError('Qubit Labels out of bound in CX Gate')
    lo, hi = min(ctl, tgt), max(ctl, tgt)
    v = np.reshape(state, (4 ** lo, 4, 4 ** (hi - lo - 1), 4, 4 ** (n - hi - 1)))
    o = v.copy()
    if ctl < tgt:
        def get(a, b):
            return o[:, a, :, b, :]

        def put(a, b, val):
            v[:, a, :, b, :] = val
    else:
        def get(a, b):
            return o[:, b, :, a, :]

        def put(a, b, val):
            v[:, b, :, a, :] = val
    # (control Pauli, target Pauli) slices
    put(0, 2, s2 * get(0, 2) + c2 * get(3, 2) - cs * (get(0, 3) - get(3, 3)))
    put(3, 2, c2 * get(0, 2) + s2 * get(3, 2) + cs * (get(0, 3) - get(3, 3)))
    put(0, 3, s2 * get(0, 3) + c2 * get(3, 3) + cs * (get(0, 2) - get(3, 2)))
    put(3, 3, c2 * get(0, 3) + s2 * get(3, 3) - cs * (get(0, 2) - get(3, 2)))
    put(1, 0, c * get(1, 1) - s * get(2, 0))
    put(1, 1, c * get(1, 0) - s * get(2, 1))
    put(1, 2, -s * get(2, 2) + c * get(2, 3))
    put(1, 3, -c * get(2, 2) - s * get(2, 3))
    put(2, 0, s * get(1, 0) + c * get(2, 1))
    put(2, 1, s * get(1, 1) + c * get(2, 0))
    put(2, 2, s * get(1, 2) - c * get(1, 3))
    put(2, 3, c * get(1, 2) + s * get(1, 3))
    return state


def memory_noise(state, n, f, p, g):
    """dm_simulator.py:397-425 (_add_decoherence_and_amp_decay): every qubit, every level."""
    k = np.sqrt(g) * f
    d = (1 - g) * (2 * p - 1)
    for q in range(n):
        v = np.reshape(state, (4 ** q, 4, 4 ** (n - q - 1)))
        old = v.copy()
        v[:, 1, :] = k * old[:, 1, :]
        v[:, 2, :] = k * old[:, 2, :]
        v[:, 3, :] = g * old[:, 3, :] + d * old[:, 0, :]
    return state


def ensemble_probabilities(state, n, basis, nvec, err):
    """dm_simulator.py:427-473 (_add_ensemble_measure), as a per-axis contraction.

    The reference forms the 2**n x 2**n Kronecker product of the per-qubit
    rows [1, +-err] (or [1, +-err*n] for basis N) and dots it with the
    gathered coefficients; contracting axis by axis gives the same sums.
    Outcome index: qubit 0 is the most significant bit.
    """
    if basis == 'N':
        w = np.asarray(nvec, dtype=float) * err
        row = np.array([[1, w[0], w[1], w[2]], [1, -w[0], -w[1], -w[2]]])
    else:
        col = {'X': 1, 'Y': 2, 'Z': 3}[basis]
        row = np.zeros((2, 4))
        row[:, 0] = 1
        row[0, col] = err
        row[1, col] = -err
    t = np.reshape(state, [4] * n)
    for q in range(n):
        t = np.tensordot(row, t, axes=([1], [q]))   # new axis 0 ...
        t = np.moveaxis(t, 0, q)                     # ... back to position q
    return np.reshape(t, 2 ** n)


def bitstring_keys(m):
    return ["".join(s) for s in itertools.product("01", repeat=m)]


def pauli_to_matrix(coeffs, n):
    """dm_simulator.py:1198-1255 (_compute_densitymatrix), vectorised.

    Per axis: (I,X,Y,Z) -> (e00, e01, e10, e11) = (I+Z, X-iY, X+iY, I-Z); then
    the per-qubit (row bit, column bit) pairs are interleaved into a
    2**n x 2**n matrix with qubit 0 as the most significant bit.
    """
    conv = np.array([[1, 0, 0, 1], [0, 1, -1j, 0], [0, 1, 1j, 0], [1, 0, 0, -1]])
    t = np.reshape(coeffs.astype(complex), [4] * n)
    for q in range(n):
        t = np.moveaxis(np.tensordot(conv, t, axes=([1], [q])), 0, q)
    t = np.reshape(t, [2, 2] * n)
    order = [2 * i for i in range(n)] + [2 * i + 1 for i in range(n)]
    return np.reshape(np.transpose(t, order), (2 ** n, 2 ** n))


# ---------------------------------------------------------------------------
# the backend  (dm_simulator.py:120-1282)
# ---------------------------------------------------------------------------

DEFAULTS = {
    "initial_densitymatrix": None,
    "chop_threshold": 1e-15,
    "thermal_factor": 1.,
    "decoherence_factor": 1.,
    "depolarization_factor": 1.,
    "bell_depolarization_factor": 1.,
    "decay_factor": 1.,
    "rotation_error": {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]},
    "tsp_model_error": [1., 0.],
}


class OracleDmSimulator:
    """Restatement of ``DmSimulatorPy`` (dm_simulator.py:61-1313), numpy on the host.

    Options are taken per instance (the reference's class-level leak of
    ``rotation_error`` updates, dm_simulator.py:182/:212-213, is not
    modelled here: each oracle instance starts from the defaults).
    """

    def __init__(self, backend_options=None, custom_densitymatrix=None):
        self.custom = custom_densitymatrix
        self.set_options(backend_options or {})

    # dm_simulator.py:177-271
    def set_options(self, opts):
        self.initial = DEFAULTS['initial_densitymatrix']
        self.chop = DEFAULTS['chop_threshold']
        self.rot_err = copy.deepcopy(DEFAULTS['rotation_error'])
        self.tsp = list(DEFAULTS['tsp_model_error'])
        self.p = DEFAULTS['thermal_factor']
        self.f = DEFAULTS['decoherence_factor']
        self.g = DEFAULTS['decay_factor']
        self.depol = DEFAULTS['depolarization_factor']
        self.bell_depol = DEFAULTS['bell_depolarization_factor']
        self.get_den_mat = True
        self.merge = True
        if 'initial_densitymatrix' in opts:
            self.initial = opts['initial_densitymatrix']
        if 'custom_densitymatrix' in opts:
            self.custom = opts['custom_densitymatrix']
        if 'rotation_error' in opts:
            re = opts['rotation_error']
            if not isinstance(re, dict) or not all(k in ('rx', 'ry', 'rz') for k in re):
                raise OracleError('Incorrect Rotation Error parameters')
            self.rot_err.update(re)
        if 'tsp_model_error' in opts:
            t = opts['tsp_model_error']
            if not isinstance(t, list) or len(t) != 2 or t[0] > 1 or t[1] > 1:
                raise OracleError('Incorrect transition model error parameter')
            self.tsp = t
        self.p = opts.get('thermal_factor', self.p)
        self.f = opts.get('decoherence_factor', self.f)
        self.g = opts.get('decay_factor', self.g)
        self.depol = opts.get('depolarization_factor', self.depol)
        # 'bell_depolarization_factor' is stored on the wrong attribute by the
        # reference (dm_simulator.py:240) and so never reaches the Bell measure.
        self.chop = opts.get('chop_threshold', self.chop)
        self.get_den_mat = opts.get('compute_densitymatrix', self.get_den_mat)
        self.merge = opts.get('merge', self.merge)

    # dm_simulator.py:284-365
    def initial_state(self, n):
        if self.initial is None:
            per = {None: [1, 0, 0, 1], 'max_mixed': [1, 0, 0, 0],
                   'uniform_superpos': [1, 1, 0, 0],
                   'thermal_state': [1, 0, 0, 2 * self.p - 1]}
            if self.custom not in per:
                raise OracleError('_custom_densitymatrix value is invalid')
            vec = np.array(per[self.custom], dtype=float)
            st = vec
            for _ in range(n - 1):
                st = np.kron(vec, st)
            return st * 0.5 ** n
        if self.custom == 'binary_string':
            bits = self.initial
            if len(bits) != n:
                raise OracleError('Wrong input binary string length')
            st = np.array([1, 0, 0, 1 if bits[0] == '0' else -1], dtype=float)
            for ch in bits[1:]:
                st = np.kron([1, 0, 0, 1 if ch == '0' else -1], st)
            return st * 0.5 ** n
        if self.custom == 'stored_density_matrix':
            st = np.load('stored_density_matrix.npy')
            if len(st) != 4 ** n:
                raise OracleError('Wrong input stored density matrix')
            return st
        raise OracleError('_custom_densitymatrix value is invalid')

    # --- per-qubit measurement updates, dm_simulator.py:574-704
    def _measure_axis(self, st, n, q, basis, err, nvec=None):
        v = np.reshape(st, (4 ** q, 4, 4 ** (n - q - 1)))
        if basis == 'X':
            v[:, 1, :] *= err
            v[:, 2, :] = 0
            v[:, 3, :] = 0
        elif basis == 'Y':
            v[:, 1, :] = 0
            v[:, 3, :] = 0
            v[:, 2, :] *= err
        elif basis == 'Z':
            v[:, 1, :] = 0
            v[:, 2, :] = 0
            v[:, 3, :] *= err
        elif basis == 'N':
            t = (nvec[0] * v[:, 1, :] + nvec[1] * v[:, 2, :] + nvec[2] * v[:, 3, :]) * err
            v[:, 1, :] = t * nvec[0]
            v[:, 2, :] = t * nvec[1]
            v[:, 3, :] = t * nvec[2]

    @staticmethod
    def _normalise(nvec):
        """dm_simulator.py:706-719."""
        norm = np.linalg.norm(nvec)
        if norm == 1:
            return nvec
        logger.warning('Given direction for the measurement was not normalised.')
        return nvec / norm

    def run_experiment(self, exp):
        """dm_simulator.py:950-1196 (run_experiment); same result-dict keys."""
        n = exp.config.n_qubits
        data = {}
        st = np.array(self.initial_state(n), dtype=float).reshape(-1)
        if self.initial is not None:                     # dm_simulator.py:351-365
            if st.size != 4 ** n:
                raise OracleError('initial densitymatrix is incorrect length')
            if st[0] != 2.0 ** (-n):
                raise OracleError('Trace of initial densitymatrix is not one')
        creg = 0
        cmem = 0
        insts = merge_single_gates(exp.instructions, n, self.merge)
        levels_list, levels = partition_levels(insts, n)
        part_measure = False
        for clock in range(levels):
            level = levels_list[clock]
            # dm_simulator.py:1006-1018: is this a same-basis partial measurement?
            for op in level:
                if op.name == 'measure':
                    basis = str(getattr(level[0], 'params', ['Z'])[0])
                    prm = getattr(op, 'params', ['Z'])
                    if str(prm[0]) in ('X', 'Y', 'Z', 'N'):
                        if str(prm[0]) == basis:
                            part_measure = True
                        else:
                            part_measure = False
                            break
                    else:
                        part_measure = False
                        continue
            # dm_simulator.py:1020-1170; iterate like the reference, which
            # removes single measurements from the list it is iterating over.
            i = 0
            while i < len(level):
                op = level[i]
                i += 1
                cond = getattr(op, 'conditional', None)
                if isinstance(cond, int):
                    if not (creg >> cond) & 1:
                        continue
                elif cond is not None:
                    mask = int(cond.mask, 16)
                    if mask > 0:
                        value = cmem & mask
                        while (mask & 1) == 0:
                            mask >>= 1
                            value >>= 1
                        if value != int(cond.val, 16):
                            continue
                if op.name in ('u1', 'u3'):
                    q = op.qubits[0]
                    v = np.reshape(st, (4 ** q, 4, 4 ** (n - q - 1)))
                    for name, ang in u_decomposition(op.name, op.params):
                        rotate(v, name, ang, self.rot_err[name])
                elif op.name == 'cx':
                    cx_apply(st, n, op.qubits[0], op.qubits[1], self.tsp)
                elif op.name == 'reset':                   # dm_simulator.py:810-823
                    q = op.qubits[0]
                    v = np.reshape(st, (4 ** q, 4, 4 ** (n - q - 1)))
                    v[:, 1, :] = 0
                    v[:, 2, :] = 0
                    v[:, 3, :] = v[:, 0, :].copy()
                elif op.name == 'barrier':
                    pass
                elif op.name == 'measure':
                    prm = getattr(op, 'params', ['Z'])
                    q = op.qubits[0]
                    kind = str(prm[0])
                    if len(prm) == 1:
                        prm.append(None)
                    single = ensemble = expect = False
                    if kind == 'Ensemble':
                        ensemble = True
                    elif kind == 'Expect':
                        expect = True
                    elif len(level) == 1 or part_measure is not True:
                        single = True
                    if single:
                        if kind in ('X', 'Y'):
                            self._measure_axis(st, n, q, kind, self.depol)
                        elif kind == 'N':
                            prm[1] = self._normalise(prm[1])
                            self._measure_axis(st, n, q, 'N', self.depol, prm[1])
                        elif kind == 'Bell':
                            pair = str(prm[1])
                            probs, red = self._bell(st, n, int(pair[0]), int(pair[1]), self.bell_depol)
                            data['bell_probabilities%s%s' % (pair[0], pair[1])] = probs
                            data['reduced_bell_densitymatrix%s%s' % (pair[0], pair[1])] = red
                        else:
                            self._measure_axis(st, n, q, 'Z', self.depol)
                        # list.remove() inside the reference's for-loop makes
                        # the iteration skip the element after this one.
                        level.remove(op)
                    elif part_measure:
                        qs = [x.qubits[0] for x in level]
                        basis = kind
                        nvec = prm[1] if kind == 'N' else None
                        data['partial_probability'] = self._partial(st, n, qs, basis, nvec)
                        break
                    elif expect:
                        data['Pauli_string_expectation'] = self._expect(st, n, str(prm[1]))
                        break
                    elif ensemble:
                        spec = prm[1]
                        if len(str(spec)) == 1:
                            basis, nvec = str(spec), None
                        elif spec[0] == 'N':
                            basis, nvec = 'N', self._normalise(np.asarray(spec[1], dtype=float))
                        else:
                            raise OracleError('unrecognised ensemble basis %r' % (spec,))
                        probs = ensemble_probabilities(st, n, basis, nvec, self.depol)
                        data['ensemble_probability'] = dict(zip(bitstring_keys(n), probs))
                        break
                elif op.name == 'bfunc':
                    raise OracleError('bfunc is not supported by the levelling pass')
                else:
                    raise OracleError('dm_simulator encountered unrecognized operation "%s"' % op.name)
            memory_noise(st, n, self.f, self.p, self.g)
        vec = st.copy()
        if self.get_den_mat:
            data['densitymatrix'] = pauli_to_matrix(st, n)
        vec[np.abs(vec) < self.chop] = 0.0
        data['coeffmatrix'] = vec
        return {'name': exp.header.name, 'number_of_clock_cycles': levels, 'data': data,
                'status': 'DONE', 'success': True}

    def _partial(self, st, n, qubits, basis, nvec):
        """dm_simulator.py:492-538 (_add_partial_measure)."""
        probs = ensemble_probabilities(st, n, basis, nvec, self.depol)
        others = tuple(sorted(set(range(n)) - set(qubits)))
        m = len(qubits)
        part = np.reshape(np.sum(np.reshape(probs, [2] * n), axis=others), 2 ** m)
        for q in qubits:
            if basis == 'N' and nvec is not None:
                self._measure_axis(st, n, q, 'N', self.depol, nvec)
            else:
                self._measure_axis(st, n, q, basis, self.depol)
        return dict(zip(bitstring_keys(m), part))

    def _expect(self, st, n, pauli):
        """dm_simulator.py:540-572 (_pauli_string_expectation)."""
        for q in range(n):
            if pauli[q] in ('X', 'Y', 'Z'):
                self._measure_axis(st, n, q, pauli[q], self.depol)
        idx = sum({'I': 0, 'X': 1, 'Y': 2, 'Z': 3}[c] * 4 ** (n - 1 - q) for q, c in enumerate(pauli))
        return st[idx] * 2 ** n

    def _bell(self, st, n, qa, qb, err):
        """dm_simulator.py:721-777 (_add_bell_basis_measure), reversed-axis view kept."""
        q1, q2 = min(qa, qb), max(qa, qb)
        v = np.reshape(st, (4 ** (n - q2 - 1), 4, 4 ** (q2 - q1 - 1), 4, 4 ** q1))
        red = np.array(v[0, :, 0, :, 0]) * 2 ** (n - 2)
        for i in range(4):
            for j in range(4):
                if i != j:
                    v[:, i, :, j, :] = 0
        for i in (1, 2, 3):
            v[:, i, :, i, :] *= err
        k = [v[0, i, 0, i, 0] * 2 ** n for i in range(4)]
        probs = [0.25 * (k[0] + k[1] - k[2] + k[3]), 0.25 * (k[0] - k[1] + k[2] + k[3]),
                 0.25 * (k[0] + k[1] + k[2] - k[3]), 0.25 * (k[0] - k[1] - k[2] - k[3])]
        return dict(zip(['Bell_1', 'Bell_2', 'Bell_3', 'Bell_4'], probs)), red
