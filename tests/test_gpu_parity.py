"""GPU parity of the drop-in backend against the reference's outputs and the oracle.

* every golden case (produced by the unmodified reference) through
  ``DmSimulatorGPU.run_experiment``: FP64 fused, FP64 one-sweep-per-op, and
  FP32 fused;
* larger seeded workloads against the CPU oracle;
* n = 14 (the 2.1 GB FP64 state of the 14-qubit workload) through
  size-independent properties.

Tolerances: FP64 paths agree with the reference to 1e-12 on the Pauli
expectations 2**n a_s and on probabilities; FP32 paths (CUDA cores and the
tensor-core FP16 split) to FP32_TOL = 1e-6 on the same values, and the L1
distance of every probability distribution to 1e-6 as well.
"""
import copy

import numpy as np
import pytest

import golden_cases as G
import qiskit_aakash_gb300 as dmg
from oracle import dm_oracle as O
from test_oracle import compare_outputs

pytestmark = pytest.mark.gpu

CASES = [c for c in G.cases() if 'error' not in c]
FP32_TOL = 1e-6      # max-abs of 2**n a_s and of probabilities, and probability L1, for FP32 results


@pytest.fixture(scope='module', autouse=True)
def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail('CUDA device required for the gpu tests')
    dmg.build()


def run_gpu(exp, opts, **extra):
    from qiskit_aakash_gb300.dm_simulator import DmSimulatorGPU
    DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    b = DmSimulatorGPU()
    o = copy.deepcopy(opts)
    o.update(extra)
    b._set_options(backend_options=o)
    res = b.run_experiment(exp)
    return res, b


@pytest.mark.parametrize('c', CASES, ids=lambda c: c['name'])
def test_golden_fp64_fused(c):
    res, _ = run_gpu(G.experiment(c), G.options(c))
    assert res['number_of_clock_cycles'] == c['number_of_clock_cycles']
    compare_outputs(c, res['data'], rel=1e-12)


@pytest.mark.parametrize('c', CASES[::3], ids=lambda c: c['name'])
def test_golden_fp64_one_sweep_per_op(c):
    res, _ = run_gpu(G.experiment(c), G.options(c), fusion=False)
    compare_outputs(c, res['data'], rel=1e-12)


@pytest.mark.parametrize('c', CASES[::2], ids=lambda c: c['name'])
def test_golden_fp32_fused(c):
    res, _ = run_gpu(G.experiment(c), G.options(c), precision='single')
    compare_outputs(c, res['data'], rel=FP32_TOL, l1=FP32_TOL)


def _oracle(exp, opts):
    return O.OracleDmSimulator(copy.deepcopy(opts)).run_experiment(copy.deepcopy(exp))


def _assert_close(a, b, n, rel):
    for k, v in b['data'].items():
        g = a['data'][k]
        if isinstance(v, dict):
            assert list(g.keys()) == list(v.keys())
            np.testing.assert_allclose(list(g.values()), list(v.values()), rtol=0, atol=rel)
            l1 = np.abs(np.array(list(g.values()), dtype=float) - np.array(list(v.values()), dtype=float)).sum()
            assert l1 <= max(rel, 1e-12 * len(v)), (k, l1)
        elif k == 'coeffmatrix':
            np.testing.assert_allclose(np.asarray(g) * 2 ** n, np.asarray(v) * 2 ** n, rtol=0, atol=rel)
        else:
            np.testing.assert_allclose(np.asarray(g), np.asarray(v), rtol=0, atol=rel)


@pytest.mark.parametrize('n,layers,seed,every_gate,qft', [
    (10, 6, 11, False, False),
    (11, 3, 12, False, False),
    (8, 2, 13, True, True),
    (9, 3, 14, True, False),
])
def test_workloads_match_oracle(n, layers, seed, every_gate, qft):
    qc = dmg.random_layer_circuit(n, layers, seed, barrier_after_gate=every_gate, qft=qft)
    opts = dmg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
    opts['compute_densitymatrix'] = False
    ref = _oracle(qc.to_experiment(), opts)
    for kw, tol in (({}, 1e-12), ({'tile_axes': 7}, 1e-12), ({'tile_axes': 4}, 1e-12),
                    ({'register_rounds': False}, 1e-12), ({'precision': 'single'}, FP32_TOL),
                    ({'precision': 'single', 'tma': False}, FP32_TOL),
                    ({'precision': 'single', 'compose': 'host'}, FP32_TOL),
                    ({'precision': 'single', 'tensor_cores': False}, FP32_TOL),
                    ({'precision': 'single', 'tensor_cores': False, 'register_rounds': False}, FP32_TOL)):
        got, b = run_gpu(qc.to_experiment(), opts, **kw)
        assert got['number_of_clock_cycles'] == ref['number_of_clock_cycles']
        _assert_close(got, ref, n, tol)


def test_fourteen_qubit_properties():
    """14 qubits (2.1 GB in FP64): QFT + 2 noisy layers, noise after every gate."""
    n = 14
    qc = dmg.random_layer_circuit(n, 2, 5, barrier_after_gate=True, qft=True)
    opts = dmg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
    opts['compute_densitymatrix'] = False
    fused, b = run_gpu(qc.to_experiment(), opts)
    a = fused['data']['coeffmatrix']
    assert a[0] == 2.0 ** -n                         # trace preserved exactly
    p = np.array(list(fused['data']['ensemble_probability'].values()))
    assert abs(p.sum() - 1.0) < 1e-12 and p.min() > -1e-12
    assert b.last_run_stats['passes'] < fused['number_of_clock_cycles']
    single, _ = run_gpu(qc.to_experiment(), opts, precision='single')
    np.testing.assert_allclose(single['data']['coeffmatrix'] * 2 ** n, a * 2 ** n, rtol=0, atol=FP32_TOL)
    cuda_cores, _ = run_gpu(qc.to_experiment(), opts, precision='single', tensor_cores=False)
    np.testing.assert_allclose(cuda_cores['data']['coeffmatrix'] * 2 ** n, a * 2 ** n, rtol=0, atol=FP32_TOL)
    for r in (single, cuda_cores):
        p32 = np.array(list(r['data']['ensemble_probability'].values()))
        assert np.abs(p32 - p).sum() <= FP32_TOL
    unfused, _ = run_gpu(qc.to_experiment(), opts, fusion=False)
    np.testing.assert_allclose(unfused['data']['coeffmatrix'] * 2 ** n, a * 2 ** n, rtol=0, atol=1e-12)


def test_execute_and_provider_path():
    """README example through BasicAer.get_backend('dm_simulator') and execute()."""
    from qiskit_aakash_gb300.dm_simulator import DmSimulatorGPU
    # rotation_error options update the class-level defaults (as in the
    # reference, dm_simulator.py:182, :212-213): start from the true defaults.
    DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    qc = dmg.QuantumCircuit(2)
    qc.x(1)
    qc.cx(0, 1)
    backend = dmg.BasicAer.get_backend('dm_simulator')
    result = dmg.execute(qc, backend).result()
    dm = result['results'][0]['data']['densitymatrix']
    expect = np.zeros((4, 4))
    expect[1, 1] = 1
    np.testing.assert_allclose(dm, expect, atol=1e-15)
    assert result['backend_name'] == 'dm_simulator' and result['success']


def test_rotation_error_defaults_leak_like_the_reference():
    """A run with rotation_error changes the defaults seen by later runs (dm_simulator.py:212-213)."""
    from qiskit_aakash_gb300.dm_simulator import DmSimulatorGPU
    DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    qc = dmg.QuantumCircuit(1)
    qc.x(0)
    backend = dmg.BasicAer.get_backend('dm_simulator')
    dmg.execute(qc, backend, rotation_error={'ry': [0.5, 0.0]}).result()
    r = dmg.execute(qc, backend).result()['results'][0]['data']['coeffmatrix']
    assert abs(r[3] - (-0.25)) < 1e-12       # Z coefficient: ry contracted by 0.5
    DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}


def test_tensor_core_round_overflow_falls_back_to_the_cuda_core_pass():
    """A pass with more rounds than a tensor-core descriptor holds runs on the CUDA cores, same result."""
    n = 7
    qc = dmg.QuantumCircuit(n, n)
    for i in range(120):                   # a CX chain around all 7 qubits, u3 in between
        qc.u3(0.1 * i, 0.2, 0.3, i % n)
        qc.cx(i % n, (i + 1) % n)
    qc.measure(list(range(n)), list(range(n)), basis='Ensemble', add_param='Z')
    opts = dmg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998)
    opts['compute_densitymatrix'] = False
    ref = _oracle(qc.to_experiment(), opts)
    got, _ = run_gpu(qc.to_experiment(), opts, precision='single')
    _assert_close(got, ref, n, FP32_TOL)


@pytest.mark.parametrize('precision', ['double', 'single'])
def test_streamed_launches_equal_one_flush(precision, monkeypatch):
    """The engine launches passes while the run loop still queues operations; with a tiny streaming
    threshold (many partial flushes) the state is bit for bit the one of launching everything at the
    first read-out, and both match the oracle."""
    from qiskit_aakash_gb300 import engine
    n = 9
    qc = dmg.random_layer_circuit(n, 4, 21, barrier_after_gate=True)
    opts = dmg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
    opts['compute_densitymatrix'] = False
    monkeypatch.setattr(engine, 'STREAM_OPS', 10 ** 9)
    whole, b1 = run_gpu(qc.to_experiment(), opts, precision=precision)
    monkeypatch.setattr(engine, 'STREAM_OPS', 40)
    streamed, b2 = run_gpu(qc.to_experiment(), opts, precision=precision)
    assert b1.last_run_stats['passes'] == b2.last_run_stats['passes']
    assert np.array_equal(whole['data']['coeffmatrix'], streamed['data']['coeffmatrix'])
    ref = _oracle(qc.to_experiment(), opts)
    _assert_close(streamed, ref, n, 1e-12 if precision == 'double' else FP32_TOL)


def test_tensor_core_fp32_against_fp64_twelve_qubits_twenty_layers():
    """12 qubits, 20 noisy layers, noise after every gate: the tensor-core FP32 form (TMA-fed and
    cp.async-fed) against the FP64 form on the GPU, at the 1e-6 bound on 2**n a_s and probability L1."""
    n = 12
    qc = dmg.random_layer_circuit(n, 20, 31, barrier_after_gate=True)
    opts = dmg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
    opts['compute_densitymatrix'] = False
    ref, _ = run_gpu(qc.to_experiment(), opts)
    a = ref['data']['coeffmatrix']
    p = np.array(list(ref['data']['ensemble_probability'].values()))
    for kw in ({}, {'tma': False}, {'compose': 'host'}):
        got, b = run_gpu(qc.to_experiment(), opts, precision='single', **kw)
        assert b.last_run_stats['passes'] > 0
        assert b.last_run_stats['composed_on'][kw.get('compose', 'device')] > 0
        err = np.abs(got['data']['coeffmatrix'] - a).max() * 2 ** n
        p32 = np.array(list(got['data']['ensemble_probability'].values()))
        assert err <= FP32_TOL, (kw, err)
        assert np.abs(p32 - p).sum() <= FP32_TOL, kw


def test_fp64_check_states_the_fp32_error():
    """precision='single' with fp64_check: the result states its max-abs coefficient error and
    probability L1 error against the same experiment in FP64 (and both are within 1e-6)."""
    n = 9
    qc = dmg.random_layer_circuit(n, 6, 41, barrier_after_gate=True)
    qc.measure([0, 3], [0, 3], basis='Ensemble', add_param='X')
    opts = dmg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
    opts['compute_densitymatrix'] = False
    got, _ = run_gpu(qc.to_experiment(), opts, precision='single', fp64_check=True)
    ref, _ = run_gpu(qc.to_experiment(), opts)
    d = got['data']
    assert 0 < d['max_abs_coeff_err'] <= FP32_TOL
    assert 0 <= d['prob_l1_err'] <= FP32_TOL
    assert d['trace_err'] <= FP32_TOL
    host_err = np.abs(d['coeffmatrix'] - ref['data']['coeffmatrix']).max() * 2 ** n
    assert abs(host_err - d['max_abs_coeff_err']) <= 1e-9
    p32 = np.array(list(d['ensemble_probability'].values()))
    p64 = np.array(list(ref['data']['ensemble_probability'].values()))
    assert np.abs(p32 - p64).sum() <= d['prob_l1_err'] + 1e-15
    plain, _ = run_gpu(qc.to_experiment(), opts, precision='single')
    assert 'max_abs_coeff_err' not in plain['data'] and 'trace_err' not in plain['data']


@pytest.mark.parametrize('precision', ['double', 'single'])
def test_trace_violation_raises(precision, monkeypatch):
    """A state whose trace coefficient left 2**-n is reported as an error after the run.

    The corruption is made on the host: before the final check reads a_0,
    the state is read back, a_0 is halved and the vector is loaded again
    through dm_load_state."""
    from qiskit_aakash_gb300 import engine
    from qiskit_aakash_gb300.exceptions import BasicAerError
    n = 8
    qc = dmg.random_layer_circuit(n, 2, 43)
    opts = dmg.noise_options(decoherence=0.99, decay=0.99)
    opts['compute_densitymatrix'] = False
    ok, _ = run_gpu(qc.to_experiment(), opts, precision=precision)
    assert ok['success']
    original = engine.DeviceState.trace_error

    def corrupted(self):
        a = self.raw_coefficients().astype(np.float64)
        a[0] *= 0.5
        self.load(a)
        return original(self)

    monkeypatch.setattr(engine.DeviceState, 'trace_error', corrupted)
    with pytest.raises(BasicAerError, match='Trace of densitymatrix is not one after the run'):
        run_gpu(qc.to_experiment(), opts, precision=precision)


@pytest.mark.parametrize('n', [13, 14])
def test_qft_workload_matches_reference_fixture(n):
    """QFT + 2 random layers with the full noise model after every gate, against the reference itself.

    tests/golden/make_c2_fixture.py ran the unmodified DmSimulatorPy on this
    circuit (a few CPU-hours at n = 14) and kept its clock cycles, all 2**n
    ensemble probabilities, every coefficient on the Z sublattice, 65,536
    coefficients at seeded random indices and checksums of the whole vector.
    FP64 on the GPU must match at 1e-12 (Pauli expectations 2**n a_s and
    probabilities); the FP32 tensor-core form at FP32_TOL."""
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'c2_qft_n%d_L2_s0.npz' % n)
    if not os.path.exists(path):
        pytest.skip('fixture %s not generated' % os.path.basename(path))
    fx = np.load(path)
    meta = json.loads(str(fx['meta']))
    qc = dmg.random_layer_circuit(n, meta['layers'], meta['seed'], barrier_after_gate=True, qft=True)
    opts = dict(meta['options'])
    for precision, tol in (('double', 1e-12), ('single', FP32_TOL)):
        got, _ = run_gpu(qc.to_experiment(), opts, precision=precision)
        assert got['number_of_clock_cycles'] == int(fx['clock_cycles'])
        a = np.asarray(got['data']['coeffmatrix'])
        p = np.array(list(got['data']['ensemble_probability'].values()))
        assert list(got['data']['ensemble_probability'].keys())[1] == '0' * (n - 1) + '1'
        np.testing.assert_allclose(p, fx['probs'], rtol=0, atol=tol)
        np.testing.assert_allclose(a[fx['z_idx'].astype(np.int64)] * 2 ** n, fx['z_val'] * 2 ** n, rtol=0, atol=tol)
        np.testing.assert_allclose(a[fx['idx'].astype(np.int64)] * 2 ** n, fx['val'] * 2 ** n, rtol=0, atol=tol)
        if precision == 'double':
            # checksums of all 4**n coefficients (each agreeing to ~1e-15 in units of 2**-n)
            assert abs(a.sum() - float(fx['coeff_sum'])) * 2 ** n <= 1e-6
            assert abs(np.abs(a).sum() - float(fx['coeff_abs_sum'])) * 2 ** n <= 1e-6
        else:
            assert np.abs(p - fx['probs']).sum() <= tol
        del a
