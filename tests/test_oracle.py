"""Pin the CPU oracle against the reference's own outputs (golden fixtures)."""
import copy

import numpy as np
import pytest

import golden_cases as G
from oracle import dm_oracle as O

ALL = G.cases()


def _signature(c):
    insts = G.instructions(c)
    merged = O.merge_single_gates(insts, c['n'], c['options'].get('merge', True))
    chained, levels = O.partition_levels(merged, c['n'])
    sig = []
    for lev in chained:
        row = []
        for op in lev:
            ent = [op.name, list(op.qubits)]
            if op.name in ('u1', 'u3'):
                ent.append([float(x) for x in op.params])
            row.append(ent)
        sig.append(row)
    return sig, levels


def _same_levels(a, b):
    assert len(a) == len(b)
    for la, lb in zip(a, b):
        assert len(la) == len(lb)
        for ea, eb in zip(la, lb):
            assert ea[0] == eb[0] and ea[1] == eb[1]
            if len(ea) > 2:
                np.testing.assert_allclose(ea[2], eb[2], rtol=0, atol=1e-12)


@pytest.mark.parametrize('c', [c for c in ALL if 'levels' in c], ids=lambda c: c['name'])
def test_levelling_matches_reference(c):
    sig, levels = _signature(c)
    assert levels == c['n_levels']
    _same_levels(sig, c['levels'])


def compare_outputs(c, data, rel=1e-12, l1=None):
    """Compare a result 'data' dict with the golden outputs of case c.

    rel bounds every value (Pauli expectations 2**n a_s, probabilities);
    l1, when given, also bounds the L1 distance of each probability dictionary."""
    n = c['n']
    scale = 2.0 ** n          # coefficients are Pauli expectations / 2**n
    for k, key in c['outputs'].items():
        ref = G.array(key)
        assert k in data, k
        got = data[k]
        if isinstance(got, dict):
            assert list(got.keys()) == c['dict_keys'][k]
            got = np.array([float(v) for v in got.values()])
            if l1 is not None:
                assert np.abs(got - ref).sum() <= l1, (k, np.abs(got - ref).sum())
        got = np.asarray(got)
        if k == 'coeffmatrix':
            np.testing.assert_allclose(got * scale, ref * scale, rtol=0, atol=rel)
        else:
            np.testing.assert_allclose(got, ref, rtol=0, atol=rel)
    if 'coeff_sum' in c:
        v = np.asarray(data['coeffmatrix'])
        assert abs(v.sum() - c['coeff_sum']) * scale <= rel * max(1.0, v.size ** 0.5)


@pytest.mark.parametrize('c', [c for c in ALL if 'error' not in c], ids=lambda c: c['name'])
def test_oracle_matches_reference(c):
    sim = O.OracleDmSimulator(G.options(c))
    res = sim.run_experiment(G.experiment(c))
    assert res['number_of_clock_cycles'] == c['number_of_clock_cycles']
    compare_outputs(c, res['data'])


def test_kat_values():
    """The README / notebook answers (dm_simulator_user_guide/features/*.ipynb)."""
    r = O.OracleDmSimulator().run_experiment(G.experiment(G.case('kat_readme')))
    dm = r['data']['densitymatrix']
    assert abs(dm[1, 1] - 1) < 1e-12 and abs(np.abs(dm).sum() - 1) < 1e-12
    r = O.OracleDmSimulator().run_experiment(G.experiment(G.case('kat_measure_n')))
    np.testing.assert_allclose(r['data']['densitymatrix'],
                               [[0.82142857, 0.10714286 - 0.21428571j],
                                [0.10714286 + 0.21428571j, 0.17857143]], atol=1e-8)
    r = O.OracleDmSimulator().run_experiment(G.experiment(G.case('kat_ghz_ensemble_x')))
    p = r['data']['ensemble_probability']
    assert all(abs(p[k] - 0.25) < 1e-12 for k in ('000', '011', '101', '110'))
    r = O.OracleDmSimulator().run_experiment(G.experiment(G.case('kat_ghz_expect_ziz')))
    assert abs(r['data']['Pauli_string_expectation'] - 1.0) < 1e-12
    r = O.OracleDmSimulator().run_experiment(G.experiment(G.case('kat_bell')))
    assert r['data']['bell_probabilities01'] == pytest.approx(
        {'Bell_1': .5, 'Bell_2': .5, 'Bell_3': 0, 'Bell_4': 0})


def test_oracle_planted_error_is_caught():
    """A mistake planted in the oracle (on the CPU) must fail the golden comparison."""
    c = G.case('layers8_s0')
    sim = O.OracleDmSimulator(G.options(c))
    orig = O.memory_noise
    try:
        O.memory_noise = lambda st, n, f, p, g: orig(st, n, f * (1 + 1e-9), p, g)
        res = sim.run_experiment(G.experiment(c))
    finally:
        O.memory_noise = orig
    with pytest.raises(AssertionError):
        compare_outputs(c, res['data'])
