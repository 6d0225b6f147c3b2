"""A small circuit builder that emits dm_simulator qobjs.

qiskit's transpiler unrolls every gate to the backend basis ``u1, u2, u3,
cx, id`` (dm_simulator.py:85; qiskit/transpiler/preset_passmanagers/
default.py:95-112) before the assembler builds the qobj.  This builder emits
the same unrolled forms directly, using the gate definitions of the
reference's standard extensions:

* h -> u2(0, pi)                       qiskit/extensions/standard/h.py:37-48
* x -> u3(pi, 0, pi)                   qiskit/extensions/standard/x.py:36-43
* y -> u3(pi, pi/2, pi/2)              qiskit/extensions/standard/y.py:34-42
* z -> u1(pi); s -> u1(pi/2); sdg -> u1(-pi/2); t -> u1(pi/4); tdg -> u1(-pi/4)
* rx(t) -> u3(t, -pi/2, pi/2); ry(t) -> u3(t, 0, 0); rz(p) -> u1(p)
* cu1(l) a,b -> u1(l/2) a; cx a,b; u1(-l/2) b; cx a,b; u1(l/2) b
                                       qiskit/extensions/standard/cu1.py:33-50
* measure(q, c, basis, add_param)      qiskit/circuit/measure.py:23-97: string
  parameters become ``sympy.Symbol`` (qiskit/circuit/instruction.py:139-141)
  and Ensemble / Expect / Bell measurements are wrapped in barriers.

It also holds the seeded workloads used by the tests and the benchmark: the
random brick-layer template and the QFT of the reference's ``circuits/qft.py``.
"""
import math

import numpy as np

from .qobj import Qobj, QobjExperiment, QobjInstruction

try:                               # string parameters are sympy Symbols in qobjs
    import sympy
    _Symbol = sympy.Symbol
except ImportError:                # pragma: no cover - sympy is a dependency of the reference
    _Symbol = str

PI = math.pi


class QuantumCircuit:
    """Record gates as unrolled qobj instructions."""

    def __init__(self, n_qubits, n_clbits=0, name='circuit0'):
        self.n_qubits = int(n_qubits)
        self.n_clbits = int(n_clbits)
        self.name = name
        self.instructions = []

    # -- basis gates --------------------------------------------------------
    def _q(self, q):
        q = int(q)
        if not 0 <= q < self.n_qubits:
            raise IndexError('qubit %d out of range' % q)
        return q

    def u1(self, lam, q):
        self.instructions.append(QobjInstruction('u1', [self._q(q)], [float(lam)]))
        return self

    def u2(self, phi, lam, q):
        self.instructions.append(QobjInstruction('u2', [self._q(q)], [float(phi), float(lam)]))
        return self

    def u3(self, theta, phi, lam, q):
        self.instructions.append(
            QobjInstruction('u3', [self._q(q)], [float(theta), float(phi), float(lam)]))
        return self

    def cx(self, ctl, tgt):
        self.instructions.append(QobjInstruction('cx', [self._q(ctl), self._q(tgt)]))
        return self

    def iden(self, q):
        self.instructions.append(QobjInstruction('id', [self._q(q)]))
        return self

    def barrier(self, *qubits):
        qs = [self._q(q) for q in qubits] or list(range(self.n_qubits))
        self.instructions.append(QobjInstruction('barrier', qs))
        return self

    def reset(self, q):
        self.instructions.append(QobjInstruction('reset', [self._q(q)]))
        return self

    # -- derived gates (unrolled as the reference's definitions) ------------
    def h(self, q):
        return self.u2(0.0, PI, q)

    def x(self, q):
        return self.u3(PI, 0.0, PI, q)

    def y(self, q):
        return self.u3(PI, PI / 2, PI / 2, q)

    def z(self, q):
        return self.u1(PI, q)

    def s(self, q):
        return self.u1(PI / 2, q)

    def sdg(self, q):
        return self.u1(-PI / 2, q)

    def t(self, q):
        return self.u1(PI / 4, q)

    def tdg(self, q):
        return self.u1(-PI / 4, q)

    def rx(self, theta, q):
        return self.u3(theta, -PI / 2, PI / 2, q)

    def ry(self, theta, q):
        return self.u3(theta, 0.0, 0.0, q)

    def rz(self, phi, q):
        return self.u1(phi, q)

    def cu1(self, lam, ctl, tgt):
        self.u1(lam / 2, ctl)
        self.cx(ctl, tgt)
        self.u1(-lam / 2, tgt)
        self.cx(ctl, tgt)
        return self.u1(lam / 2, tgt)

    # -- measurement (qiskit/circuit/measure.py:23-97) ----------------------
    def measure(self, qubit, cbit, basis=None, add_param=None):
        avail = ('I', 'X', 'Y', 'Z', 'N', 'Bell', 'Ensemble', 'Expect')
        if basis == 'N':
            if add_param is None:
                raise ValueError('Direction should be provided with this measurement basis.')
            params = [_Symbol('N'), np.asarray(add_param, dtype=float)]
        elif basis == 'Bell':
            if add_param is None:
                raise ValueError('Bell measurement should be provided with two qubit locations')
            params = [_Symbol('Bell'), _Symbol(str(add_param))]
        elif basis == 'Ensemble':
            params = [_Symbol('Ensemble'), _ensemble_param(add_param)]
        elif basis == 'Expect':
            if add_param is None:
                raise ValueError('Expectation measurement should be provided with string of Pauli operators')
            params = [_Symbol('Expect'), _Symbol(str(add_param))]
        elif basis is not None and add_param is None:
            if basis[0] not in avail:
                raise ValueError('Invalid basis provided.')
            params = [_Symbol(basis[0])]
        elif basis is not None:
            raise ValueError('Direction cannot be provided with this measurement basis.')
        else:
            params = None
        qubits = [qubit] if isinstance(qubit, int) else list(qubit)
        cbits = [cbit] if isinstance(cbit, int) else list(cbit)
        if len(cbits) == len(qubits):
            pairs = list(zip(qubits, cbits))
        elif len(qubits) == 1 and cbits:
            pairs = [(qubits[0], c) for c in cbits]
        else:
            raise ValueError('register size error')
        wrap = basis in ('Ensemble', 'Expect', 'Bell')
        if wrap:
            self.barrier()
        for q, c in pairs:
            self.instructions.append(QobjInstruction(
                'measure', [self._q(q)], None if params is None else list(params), [int(c)]))
        if wrap:
            self.barrier()
        return self

    # -- qobj ----------------------------------------------------------------
    def to_experiment(self, copy=True):
        """The circuit as a qobj experiment; ``copy=False`` hands over the instructions
        themselves (for a circuit that is not used again)."""
        insts = [_clone(i) for i in self.instructions] if copy else list(self.instructions)
        return QobjExperiment(insts, self.n_qubits, self.n_clbits, name=self.name)

    def to_qobj(self):
        return Qobj([self.to_experiment()])


def _ensemble_param(add_param):
    if add_param is None:
        return _Symbol('Z')
    if isinstance(add_param, str):
        return _Symbol(add_param)
    # ['N', direction]
    return [add_param[0], np.asarray(add_param[1], dtype=float)]


def _clone(inst):
    out = QobjInstruction(inst.name)
    for k, v in inst.__dict__.items():
        if isinstance(v, list):
            v = [x.copy() if isinstance(x, np.ndarray) else (list(x) if isinstance(x, list) else x)
                 for x in v]
        setattr(out, k, v)
    return out


# ---------------------------------------------------------------------------
# seeded workloads
# ---------------------------------------------------------------------------

def random_layer_angles(n, layers, seed):
    """U3 angles (theta, phi, lambda) per (layer, qubit): uniform in [0, 2 pi)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 2 * PI, size=(layers, n, 3))


def add_random_layers(qc, layers, seed, barrier_after_gate=False, first_layer=0):
    """Random brick layers: U3 on every qubit, then CX on (a, a+1) for a = L%2, L%2+2, ..."""
    n = qc.n_qubits
    ang = random_layer_angles(n, layers, seed)
    for L in range(layers):
        for q in range(n):
            qc.u3(ang[L, q, 0], ang[L, q, 1], ang[L, q, 2], q)
            if barrier_after_gate:
                qc.barrier()
        for a in range((first_layer + L) % 2, n - 1, 2):
            qc.cx(a, a + 1)
            if barrier_after_gate:
                qc.barrier()
    return qc


def add_qft(qc, barrier_after_gate=False):
    """QFT on all qubits as the general loop of the reference's circuits/qft.py:35-39."""
    n = qc.n_qubits

    def gen(k):
        return (PI * 2) / (2 ** k)

    def after():
        if barrier_after_gate:
            qc.barrier()

    for wire in range(n - 1):
        qc.h(wire)
        after()
        for rot in range(wire + 1):
            lam = gen(wire + 2 - rot)
            # cu1 unrolled; a barrier after each of its five basis gates
            qc.u1(lam / 2, wire + 1); after()
            qc.cx(wire + 1, rot); after()
            qc.u1(-lam / 2, rot); after()
            qc.cx(wire + 1, rot); after()
            qc.u1(lam / 2, rot); after()
    qc.h(n - 1)
    after()
    return qc


def random_layer_circuit(n, layers, seed, barrier_after_gate=False, measure=True, qft=False):
    """The seeded layered workload; ends with an Ensemble Z measurement of all qubits."""
    qc = QuantumCircuit(n, n, name='layers_n%d_L%d_s%d' % (n, layers, seed))
    if qft:
        add_qft(qc, barrier_after_gate)
    add_random_layers(qc, layers, seed, barrier_after_gate)
    if measure:
        qc.measure(list(range(n)), list(range(n)), basis='Ensemble', add_param='Z')
    return qc


def noise_options(depolarisation=None, decoherence=None, decay=None, rotation_sigma=None,
                  thermal=None, tsp=None):
    """Map physical noise figures onto the reference's backend options.

    depolarisation p -> depolarization_factor = 1 - p (acts at measurement,
    dm_simulator.py:281); rotation error with Gaussian sigma -> the averaged
    <cos(delta)> = exp(-sigma**2 / 2) with zero mean (basicaertools.py:93-107).
    """
    opts = {}
    if depolarisation is not None:
        opts['depolarization_factor'] = 1.0 - depolarisation
    if decoherence is not None:
        opts['decoherence_factor'] = decoherence
    if decay is not None:
        opts['decay_factor'] = decay
    if thermal is not None:
        opts['thermal_factor'] = thermal
    if rotation_sigma is not None:
        c = math.exp(-0.5 * rotation_sigma ** 2)
        opts['rotation_error'] = {'rx': [c, 0.0], 'ry': [c, 0.0], 'rz': [c, 0.0]}
    if tsp is not None:
        opts['tsp_model_error'] = list(tsp)
    return opts
