"""Generate the golden fixtures by running the reference's own dm_simulator.

Run once where the reference tree is checked out, with ``DM_REFERENCE_ROOT``
pointing at it::

    DM_REFERENCE_ROOT=<reference tree> python tests/golden/make_golden.py

It loads the unmodified ``dm_simulator.py`` / ``basicaertools.py`` through
``oracle/refload.py`` and records, for every case:

* the input (instructions, qubit count, backend options) in ``cases.json``;
* the reference's level structure (``single_gate_merge`` + ``partition``)
  and ``number_of_clock_cycles``;
* its outputs (``coeffmatrix``, ``densitymatrix`` for small n, ensemble /
  partial probabilities, Pauli-string expectation, Bell data) in
  ``outputs.npz``, or the exception it raised.

Cases: the known answers of the reference's README and user-guide notebooks,
seeded random circuits over the whole instruction set and option set
(n <= 5), the 8-qubit / 20-layer noisy brick workload for seeds 0..9, and a
5-qubit QFT + 2 layers with noise after every gate.
"""
import copy
import importlib.util
import json
import math
import os
import sys
import traceback

import numpy as np
import sympy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

from oracle import dm_oracle, refload  # noqa: E402


def _load_pkg():
    d = os.path.join(REPO, 'qiskit-aakash_gb300')
    spec = importlib.util.spec_from_file_location('qiskit_aakash_gb300', os.path.join(d, '__init__.py'),
                                                  submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules['qiskit_aakash_gb300'] = m
    spec.loader.exec_module(m)
    return m


PKG = _load_pkg()
QuantumCircuit = PKG.QuantumCircuit
S = sympy.Symbol
PI = math.pi


# ---------------------------------------------------------------------------
# (de)serialisation of instructions
# ---------------------------------------------------------------------------

def enc_param(p):
    if isinstance(p, sympy.Symbol):
        return {'s': p.name}
    if isinstance(p, np.ndarray):
        return {'a': [float(x) for x in p]}
    if isinstance(p, (list, tuple)):
        return {'l': [enc_param(x) for x in p]}
    if isinstance(p, str):
        return {'str': p}
    return {'f': float(p)}


def enc_inst(i):
    d = {'name': i.name}
    for k in ('qubits', 'memory', 'register'):
        if hasattr(i, k):
            d[k] = list(getattr(i, k))
    if hasattr(i, 'conditional'):
        d['conditional'] = i.conditional
    if hasattr(i, 'params'):
        d['params'] = [enc_param(p) for p in i.params]
    return d


# ---------------------------------------------------------------------------
# cases
# ---------------------------------------------------------------------------

CASES = []


def add(name, qc, options=None, tags=()):
    CASES.append({'name': name, 'n': qc.n_qubits, 'memory_slots': qc.n_clbits,
                  'instructions': qc.instructions, 'options': options or {}, 'tags': list(tags)})


def kat_cases():
    qc = QuantumCircuit(2, name='readme')
    qc.x(1).cx(0, 1)
    add('kat_readme', qc, tags=['kat'])
    qc = QuantumCircuit(1)
    add('kat_init_max_mixed', qc, {'custom_densitymatrix': 'max_mixed'}, tags=['kat'])
    qc = QuantumCircuit(2)
    add('kat_init_binary_01', qc, {'custom_densitymatrix': 'binary_string',
                                   'initial_densitymatrix': '01'}, tags=['kat'])
    qc = QuantumCircuit(1, 1)
    qc.s(0).measure(0, 0, basis='X')
    add('kat_measure_x', qc, tags=['kat'])
    qc = QuantumCircuit(1, 1)
    qc.s(0).measure(0, 0, basis='N', add_param=np.array([1, 2, 3]))
    add('kat_measure_n', qc, tags=['kat'])
    qc = QuantumCircuit(3, 2)
    qc.measure(0, 0, basis='Bell', add_param='01')
    add('kat_bell', qc, tags=['kat'])
    qc = QuantumCircuit(3, 3)
    qc.h(0).cx(0, 1).cx(1, 2).measure(0, 0, basis='Ensemble', add_param='X')
    add('kat_ghz_ensemble_x', qc, tags=['kat'])
    qc = QuantumCircuit(3, 3)
    qc.h(0).cx(0, 1).cx(1, 2).measure(0, 0, basis='Expect', add_param='ZIZ')
    add('kat_ghz_expect_ziz', qc, tags=['kat'])
    # features/noise.ipynb circuit, with and without its noise options
    for tag, opts in (('clean', {}), ('noisy', {
            'thermal_factor': 0., 'decoherence_factor': .9, 'depolarization_factor': 0.99,
            'bell_depolarization_factor': 0.99, 'decay_factor': 0.99,
            'rotation_error': {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]},
            'tsp_model_error': [1., 0.]})):
        qc = QuantumCircuit(3, 3)
        qc.u1(3.6, 0).cx(0, 1).u1(2.6, 2).cx(1, 0).s(2).y(2)
        qc.measure([0, 1, 2], [0, 1, 2], basis='Ensemble', add_param='Z')
        add('kat_noise_nb_' + tag, qc, opts, tags=['kat'])
    # features/partition.ipynb circuits
    qc = QuantumCircuit(3, 3)
    qc.u1(3.6, 0).cx(0, 1).u1(2.6, 2).cx(1, 0).s(2).y(2)
    add('kat_partition_1', qc, tags=['kat'])
    qc = QuantumCircuit(3, 3)
    qc.u1(3.6, 0).cx(0, 1).u1(2.6, 2)
    qc.measure(1, 1, basis='X').measure(0, 0, basis='Y')
    qc.cx(1, 0).s(2).y(2)
    qc.measure(1, 1, basis='Bell', add_param='12')
    qc.measure(0, 0)
    qc.measure([0, 1, 2], [0, 1, 2], basis='Ensemble', add_param='X')
    add('kat_partition_2', qc, tags=['kat'])


def random_circuit(rng, n, m):
    qc = QuantumCircuit(n, n)
    for _ in range(m):
        r = rng.random()
        q = int(rng.integers(n))
        if r < 0.14:
            qc.u1(rng.uniform(-PI, 3 * PI), q)
        elif r < 0.24:
            qc.u2(rng.uniform(0, 2 * PI), rng.uniform(0, 2 * PI), q)
        elif r < 0.40:
            qc.u3(rng.uniform(0, 2 * PI), rng.uniform(0, 2 * PI), rng.uniform(0, 2 * PI), q)
        elif r < 0.43:
            qc.instructions.append(PKG.QobjInstruction('U', [q], [rng.uniform(0, PI), 0.3, 0.7]))
        elif r < 0.45:
            qc.iden(q)
        elif r < 0.62 and n >= 2:
            a, b = rng.choice(n, 2, replace=False)
            qc.cx(int(a), int(b))
        elif r < 0.72:
            basis = [None, 'X', 'Y', 'Z', 'N'][int(rng.integers(5))]
            k = int(rng.integers(1, n + 1))
            qs = [int(x) for x in rng.choice(n, k, replace=False)]
            for qq in qs:
                b = basis if rng.random() < 0.8 else ['X', 'Y', 'Z'][int(rng.integers(3))]
                if b == 'N':
                    v = rng.normal(size=3)
                    if rng.random() < 0.5:
                        v = v / np.linalg.norm(v)
                    qc.measure(qq, qq, basis='N', add_param=v)
                else:
                    qc.measure(qq, qq, basis=b)
        elif r < 0.77:
            qc.reset(q)
        elif r < 0.82:
            qc.barrier()
        elif r < 0.88:
            b = ['Z', 'X', 'Y', 'N'][int(rng.integers(4))]
            if b == 'N':
                qc.measure(q, q, basis='Ensemble', add_param=['N', rng.normal(size=3)])
            else:
                qc.measure(q, q, basis='Ensemble', add_param=b)
        elif r < 0.93:
            s = ''.join('IXYZ'[int(x)] for x in rng.integers(4, size=n))
            qc.measure(q, q, basis='Expect', add_param=s)
        elif n >= 2:
            a, b = rng.choice(n, 2, replace=False)
            qc.measure(q, q, basis='Bell', add_param='%d%d' % (a, b))
    return qc


def random_options(rng):
    opts = {}
    if rng.random() < 0.6:
        opts['decoherence_factor'] = float(rng.uniform(0.85, 1.0))
    if rng.random() < 0.6:
        opts['decay_factor'] = float(rng.uniform(0.85, 1.0))
    if rng.random() < 0.4:
        opts['thermal_factor'] = float(rng.uniform(0.0, 1.0))
    if rng.random() < 0.5:
        opts['depolarization_factor'] = float(rng.uniform(0.9, 1.0))
    if rng.random() < 0.2:
        opts['bell_depolarization_factor'] = 0.9
    if rng.random() < 0.4:
        opts['rotation_error'] = {k: [float(rng.uniform(0.95, 1.0)), float(rng.uniform(-0.05, 0.05))]
                                  for k in ('rx', 'ry', 'rz') if rng.random() < 0.8}
    if rng.random() < 0.4:
        opts['tsp_model_error'] = [float(rng.uniform(0.95, 1.0)), float(rng.uniform(-0.1, 0.1))]
    if rng.random() < 0.15:
        opts['merge'] = False
    if rng.random() < 0.15:
        opts['custom_densitymatrix'] = ['max_mixed', 'uniform_superpos', 'thermal_state'][int(rng.integers(3))]
    return opts


def fuzz_cases(count=160, seed=1234):
    rng = np.random.default_rng(seed)
    for k in range(count):
        n = int(rng.integers(1, 6))
        m = int(rng.integers(1, 26))
        qc = random_circuit(rng, n, m)
        opts = random_options(rng)
        if rng.random() < 0.1:
            opts['custom_densitymatrix'] = 'binary_string'
            opts['initial_densitymatrix'] = ''.join('01'[int(x)] for x in rng.integers(2, size=n))
        add('fuzz_%03d' % k, qc, opts, tags=['fuzz'])


def workload_cases():
    for seed in range(10):
        qc = PKG.random_layer_circuit(8, 20, seed)
        opts = PKG.noise_options(depolarisation=1e-3, decoherence=0.99, decay=0.99)
        opts['compute_densitymatrix'] = False
        add('layers8_s%d' % seed, qc, opts, tags=['workload'] + (['full'] if seed < 2 else []))
    qc = PKG.random_layer_circuit(5, 2, 7, barrier_after_gate=True, qft=True)
    opts = PKG.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
    add('qft5_layers2_noise_every_gate', qc, opts, tags=['workload', 'full'])
    qc = PKG.random_layer_circuit(6, 6, 3)
    opts = PKG.noise_options(depolarisation=1e-3, decoherence=0.99, decay=0.98, thermal=0.8,
                             rotation_sigma=3e-2, tsp=[0.97, 0.02])
    add('layers6_all_noise', qc, opts, tags=['workload', 'full'])


# ---------------------------------------------------------------------------
# run through the reference
# ---------------------------------------------------------------------------

def level_signature(dm, insts, n, merge):
    merged = dm.single_gate_merge(copy.deepcopy(insts), n, merge)
    chained, levels = dm.partition(merged, n)
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


def run_case(dm, case):
    dm.DmSimulatorPy.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    n = case['n']
    insts = case['instructions']
    opts = case['options']
    out = {}
    # refuse cases on which the reference's levelling would spin forever
    try:
        dm_oracle.partition_levels(dm_oracle.merge_single_gates(copy.deepcopy(insts), n,
                                                                opts.get('merge', True)), n)
    except dm_oracle.OracleError as e:
        if 'no progress' in str(e):
            return None
    try:
        sig, levels = level_signature(dm, insts, n, opts.get('merge', True))
        out['levels'] = sig
        out['n_levels'] = levels
    except Exception as e:  # noqa: BLE001
        out['error'] = '%s: %s' % (type(e).__name__, e)
        return out
    backend = dm.DmSimulatorPy()
    exp = PKG.QobjExperiment(copy.deepcopy(insts), n, case['memory_slots'], name=case['name'])
    try:
        backend._set_options(qobj_config=None, backend_options=copy.deepcopy(opts))
        res = backend.run_experiment(exp)
    except Exception as e:  # noqa: BLE001
        out['error'] = '%s: %s' % (type(e).__name__, str(e).split('\n')[0][:200])
        return out
    out['number_of_clock_cycles'] = res['number_of_clock_cycles']
    out['data'] = res['data']
    return out


def main():
    dm = refload.load()
    kat_cases()
    fuzz_cases()
    workload_cases()
    meta = []
    arrays = {}
    n_err = 0
    for case in CASES:
        out = run_case(dm, case)
        if out is None:
            continue
        rec = {'name': case['name'], 'n': case['n'], 'memory_slots': case['memory_slots'],
               'tags': case['tags'], 'options': case['options'],
               'instructions': [enc_inst(i) for i in case['instructions']]}
        if 'levels' in out:
            rec['levels'] = out['levels']
            rec['n_levels'] = out['n_levels']
        if 'error' in out:
            rec['error'] = out['error']
            n_err += 1
            meta.append(rec)
            continue
        rec['number_of_clock_cycles'] = out['number_of_clock_cycles']
        data = out['data']
        keys = {}
        full = case['n'] <= 5 or 'full' in case['tags']
        for k, v in data.items():
            key = '%s/%s' % (case['name'], k)
            if k == 'coeffmatrix':
                v = np.asarray(v, dtype=float)
                rec['coeff_sum'] = float(np.sum(v))
                rec['coeff_abs_sum'] = float(np.sum(np.abs(v)))
                if full:
                    arrays[key] = v
                    keys[k] = key
            elif k == 'densitymatrix':
                if case['n'] <= 3:
                    arrays[key] = np.asarray(v)
                    keys[k] = key
            elif isinstance(v, dict):
                rec.setdefault('dict_keys', {})[k] = list(v.keys())
                arrays[key] = np.array([float(x) for x in v.values()])
                keys[k] = key
            else:
                arrays[key] = np.asarray(v, dtype=float)
                keys[k] = key
        rec['outputs'] = keys
        meta.append(rec)
    with open(os.path.join(HERE, 'cases.json'), 'w') as f:
        json.dump({'generator': 'tests/golden/make_golden.py', 'cases': meta}, f, indent=0)
    np.savez_compressed(os.path.join(HERE, 'outputs.npz'), **arrays)
    print('cases: %d (reference raised on %d)' % (len(meta), n_err))


if __name__ == '__main__':
    try:
        main()
    except Exception:
        traceback.print_exc()
        sys.exit(1)
