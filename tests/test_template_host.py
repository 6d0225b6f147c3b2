"""Host side of template (parametric) batched programs (no GPU).

The recipe tables are replayed with numpy exactly as the kernel composes
them (FP64, per slot, from an instance's parameter vector) and the passes
applied; the Z probabilities must equal the oracle's run of the same
template with that instance's noise options."""
import math

import numpy as np
import pytest

from oracle import dm_oracle as O
from qiskit_aakash_gb300 import _native as N
from qiskit_aakash_gb300 import template as TP
from qiskit_aakash_gb300.circuit import noise_options, random_layer_circuit

from test_planner import apply_map1, apply_pair, cx_matrix

_PLANES = {0: (2, 3), 1: (3, 1), 2: (1, 2)}


def compose(prog, slot, prm):
    b, ln = prog.slots[slot].begin, prog.slots[slot].len
    first = prog.recipes[int(prog.chain[b])]
    if first.kind == N.DM_RECIPE_CX:
        cav, mean = prm[9], prm[10]
        c2av = 4 * cav - 3
        return np.array([cav * math.cos(mean), cav * math.sin(mean), 0.5 * (1 + c2av * math.cos(2 * mean)),
                         0.5 * (1 - c2av * math.cos(2 * mean)), c2av * math.sin(mean) * math.cos(mean)])
    m = np.eye(4)
    for c in range(ln):
        r = prog.recipes[int(prog.chain[b + c])]
        if r.kind == N.DM_RECIPE_ROT:
            for k in range(r.nrot):
                ax = r.axis[k]
                k0, k1 = _PLANES[ax]
                e0, e1 = prm[3 + 2 * ax], prm[4 + 2 * ax]
                R = np.eye(4)
                cc, ss = e0 * math.cos(r.angle[k] + e1), e0 * math.sin(r.angle[k] + e1)
                R[k0, k0], R[k0, k1], R[k1, k0], R[k1, k1] = cc, -ss, ss, cc
                m = R @ m
        elif r.kind == N.DM_RECIPE_NOISE:
            f, p, g = prm[0], prm[1], prm[2]
            Nm = np.diag([1.0, math.sqrt(g) * f, math.sqrt(g) * f, g])
            Nm[3, 0] = (1 - g) * (2 * p - 1)
            m = Nm @ m
        else:
            C = prog.consts[r.const_off:r.const_off + 16]
            m = C.reshape(4, 4) @ m if ln > 1 else C.reshape(4, 4)
    return m.reshape(16)


def emulate(prog, prm):
    n = prog.n
    st = np.zeros(4 ** n)
    for i in range(2 ** n):
        st[sum(3 * 4 ** q for q in range(n) if (i >> q) & 1)] = 2.0 ** -n
    slot = 0
    for p in range(prog.npasses):
        bp = prog.passes[p]
        if isinstance(bp, N.DmBatchTcPass):
            bp = bp.ops
            assert all(bp.ops[o].moff == 16 * o for o in range(bp.nops))
        axes = [bp.axes[r] for r in range(bp.k)]
        for o in range(bp.nops):
            d = bp.ops[o]
            coef = compose(prog, slot + o, prm)
            qa = axes[d.a]
            if d.kind == N.DM_OP_MAP1:
                if d.flags & N.DM_MAP1_ROW0_IDENTITY:
                    assert coef[0] == 1.0 and not coef[1:4].any()
                st = apply_map1(st, n, qa, coef.reshape(4, 4))
            elif d.kind == N.DM_OP_CX:
                st = apply_pair(st, n, qa, axes[d.b], cx_matrix(coef, False))
            else:
                st = apply_pair(st, n, qa, axes[d.b], np.diag(coef))
        slot += bp.nops
    assert slot == prog.nslots
    return O.ensemble_probabilities(st, n, 'Z', None, prm[11])


def instance_options(rng):
    return noise_options(depolarisation=10 ** rng.uniform(-4, -2), decoherence=1 - 10 ** rng.uniform(-4, -2),
                         decay=1 - 10 ** rng.uniform(-4, -2), thermal=rng.uniform(0.8, 1.0),
                         rotation_sigma=rng.uniform(0, 0.05), tsp=[1 - 10 ** rng.uniform(-4, -2), 0.0])


@pytest.mark.parametrize('precision,n,layers', [('single', 5, 4), ('double', 4, 6), ('single', 3, 3)])
def test_template_program_replay_equals_oracle(precision, n, layers):
    rng = np.random.default_rng(n * 100 + layers)
    qc = random_layer_circuit(n, layers, seed=7)
    prog = TP.TemplateProgram(qc.to_experiment(), instance_options(rng), precision)
    for _ in range(3):
        opts = instance_options(rng)
        prm = TP.param_vector(opts)
        want = O.OracleDmSimulator(dict(opts, compute_densitymatrix=False)).run_experiment(qc.to_experiment())
        want = np.array([want['data']['ensemble_probability'][k] for k in O.bitstring_keys(n)])
        assert np.max(np.abs(emulate(prog, prm) - want)) < 1e-12


def test_tensor_core_template_program_replay_equals_oracle():
    """FP32 templates of >= 9 qubits are planned for the tensor cores (7 resident axes, rounds in
    their layouts' digit order, op o of a pass on coefficient slot o)."""
    n, layers = 9, 3
    rng = np.random.default_rng(77)
    qc = random_layer_circuit(n, layers, seed=3)
    prog = TP.TemplateProgram(qc.to_experiment(), instance_options(rng), 'single')
    assert prog.tc and isinstance(prog.passes[0], N.DmBatchTcPass)
    assert not TP.TemplateProgram(qc.to_experiment(), instance_options(rng), 'single', tensor_cores=False).tc
    for _ in range(2):
        opts = instance_options(rng)
        prm = TP.param_vector(opts)
        want = O.OracleDmSimulator(dict(opts, compute_densitymatrix=False)).run_experiment(qc.to_experiment())
        want = np.array([want['data']['ensemble_probability'][k] for k in O.bitstring_keys(n)])
        assert np.max(np.abs(emulate(prog, prm) - want)) < 1e-12


def test_template_rejects_structure_that_depends_on_parameters():
    qc = random_layer_circuit(4, 3, seed=1)
    # no memory noise in the recording: the noise maps are skipped, so the structure differs
    with pytest.raises(Exception):
        TP.TemplateProgram(qc.to_experiment(), {}, 'single')


def test_param_vector_defaults_and_mapping():
    v = TP.param_vector({})
    assert list(v[:12]) == [1, 1, 1, 1, 0, 1, 0, 1, 0, 1, 0, 1]
    v = TP.param_vector(noise_options(depolarisation=0.01, decoherence=0.99, decay=0.98, thermal=0.9,
                                      rotation_sigma=0.1, tsp=[0.97, 0.02]))
    assert np.allclose(v[:12], [0.99, 0.9, 0.98] + [math.exp(-0.005), 0] * 3 + [0.97, 0.02, 0.99])


def test_tensor_core_template_choice_is_rejected_where_it_cannot_run():
    rng = np.random.default_rng(3)
    qc = random_layer_circuit(5, 2, seed=2)
    with pytest.raises(Exception):
        TP.TemplateProgram(qc.to_experiment(), instance_options(rng), 'single', tensor_cores=True)
    qc9 = random_layer_circuit(9, 2, seed=2)
    assert not TP.TemplateProgram(qc9.to_experiment(), instance_options(rng), 'double').tc
    with pytest.raises(Exception):
        TP.TemplateProgram(qc9.to_experiment(), instance_options(rng), 'double', tensor_cores=True)
