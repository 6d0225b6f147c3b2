"""The product's merge + levelling against the reference's level structure."""
import numpy as np
import pytest

import golden_cases as G
from qiskit_aakash_gb300 import scheduler as S

ALL = [c for c in G.cases() if 'levels' in c]


@pytest.mark.parametrize('c', ALL, ids=lambda c: c['name'])
def test_levels_match_reference(c):
    insts = G.instructions(c)
    merged = S.merge_single_gates(insts, c['n'], c['options'].get('merge', True))
    table, levels = S.levelize(merged, c['n'])
    assert levels == c['n_levels']
    assert len(table) == len(c['levels'])
    for got, ref in zip(table, c['levels']):
        assert [[op.name, list(op.qubits)] for op in got] == [r[:2] for r in ref]
        for op, r in zip(got, ref):
            if len(r) > 2:
                np.testing.assert_allclose([float(x) for x in op.params], r[2], rtol=0, atol=1e-12)


def test_euler_conversion_is_a_rotation_identity():
    rng = np.random.default_rng(5)

    def rz(a):
        return np.array([[np.exp(-0.5j * a), 0], [0, np.exp(0.5j * a)]])

    def ry(a):
        return np.array([[np.cos(a / 2), -np.sin(a / 2)], [np.sin(a / 2), np.cos(a / 2)]])

    for _ in range(200):
        xi, t1, t2 = rng.uniform(0, 2 * np.pi, 3)
        beta, alpha, gamma = S.euler_zyz_from_yzy(xi, t1, t2)
        lhs = ry(t1) @ rz(xi) @ ry(t2)
        rhs = rz(alpha) @ ry(beta) @ rz(gamma)
        # equal up to a global sign
        assert min(np.abs(lhs - rhs).max(), np.abs(lhs + rhs).max()) < 1e-9


def test_compiled_levelling_rejects_what_the_reference_cannot_level():
    """dm_levelize: an instruction that can never be placed, and malformed arrays."""
    import ctypes
    from qiskit_aakash_gb300 import _native as N
    from qiskit_aakash_gb300.circuit import QobjInstruction
    from qiskit_aakash_gb300.exceptions import QiskitError
    with pytest.raises(QiskitError, match='cannot place'):
        S.levelize([QobjInstruction('u3', [0], [0.1, 0.2, 0.3]), QobjInstruction('unitary', [1], [])], 2)
    kind = np.array([N.DM_SCHED_GATE1], dtype=np.int32)
    qoff = np.array([0, 1], dtype=np.int32)
    bad_q = np.array([5], dtype=np.int32)                 # qubit beyond n
    out = np.zeros(8, dtype=np.int32)

    def p(a):
        return ctypes.c_void_p(a.ctypes.data)

    rc = N.lib().dm_levelize(2, 1, p(kind), p(qoff), p(bad_q), p(out), p(out), p(out), p(out), p(out))
    assert rc == N.DM_ERR_ARG
    assert S.levelize([], 3) == ([], 0)
