"""Generate the n=14 QFT + random-layer fixture by running the reference itself.

The workload: a QFT on all n qubits (unrolled as the transpiler does:
h -> u2(0, pi), cu1 -> u1, cx, u1, cx, u1), then random brick layers, a
barrier after every gate so that the reference's per-level memory noise
follows every gate, full noise (depolarisation 1e-3 at measurement,
decoherence 0.995, amplitude decay 0.998, rotation error sigma 1e-3 rad) and an
Ensemble Z measurement of all qubits.  ``DmSimulatorPy.run_experiment``
(qiskit/providers/basicaer/dm_simulator.py:950-1196) runs it unmodified through
``oracle/refload.py``; at n=14 that is a few CPU-hours.

Run where the reference tree is checked out::

    DM_REFERENCE_ROOT=<reference tree> python tests/golden/make_c2_fixture.py [n] [layers] [seed]

Writes ``tests/golden/c2_qft_n{n}_L{layers}_s{seed}.npz``:

* ``probs``: the 2^n ensemble probabilities, bit string order of the result
  dictionary (qubit 0 first);
* ``z_idx``/``z_val``: every coefficient whose Pauli labels are only I and Z
  (the 2^n entries the Z probabilities are built from);
* ``idx``/``val``: 65,536 coefficients at seeded random indices;
* ``coeff_sum``/``coeff_abs_sum``: checksums of the whole 4^n vector;
* ``clock_cycles``, ``n_levels`` and a JSON ``meta`` string (options, timing).
"""
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import refload  # noqa: E402

SAMPLES = 65536


def load_pkg():
    d = os.path.join(REPO, 'qiskit-aakash_gb300')
    spec = importlib.util.spec_from_file_location('qiskit_aakash_gb300', os.path.join(d, '__init__.py'),
                                                  submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules['qiskit_aakash_gb300'] = m
    spec.loader.exec_module(m)
    return m


def c2_case(pkg, n, layers, seed):
    """The circuit and backend options of the QFT + layers workload."""
    qc = pkg.random_layer_circuit(n, layers, seed, barrier_after_gate=True, qft=True)
    opts = pkg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
    opts['compute_densitymatrix'] = False
    return qc, opts


def z_sublattice(n):
    """Flat indices of the coefficients with only I (0) or Z (3) labels, bit b of k -> qubit b."""
    idx = np.zeros(1 << n, dtype=np.int64)
    for q in range(n):
        bit = (np.arange(1 << n) >> (n - 1 - q)) & 1
        idx += bit * 3 * 4 ** (n - 1 - q)
    return idx


def sample_indices(n, seed):
    rng = np.random.default_rng(1000 + seed)
    return np.unique(np.concatenate([[0], rng.integers(0, 4 ** n, size=SAMPLES)]))


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 14
    layers = int(sys.argv[2]) if len(sys.argv) > 2 else 2
    seed = int(sys.argv[3]) if len(sys.argv) > 3 else 0
    pkg = load_pkg()
    dm = refload.load()
    dm.DmSimulatorPy.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    qc, opts = c2_case(pkg, n, layers, seed)
    backend = dm.DmSimulatorPy()
    backend._set_options(qobj_config=None, backend_options=dict(opts))

    # progress only: count the per-level noise calls, then call the reference's own method
    inner = backend._add_decoherence_and_amp_decay
    t0 = time.time()
    count = [0]

    def counted(*a, **k):
        count[0] += 1
        if count[0] % 10 == 0:
            print('level %d  %.0f s' % (count[0], time.time() - t0), flush=True)
        return inner(*a, **k)

    backend._add_decoherence_and_amp_decay = counted
    res = backend.run_experiment(qc.to_experiment())
    wall = time.time() - t0
    d = res['data']
    coeff = np.asarray(d['coeffmatrix'], dtype=np.float64).ravel()
    probs = np.array([float(v) for v in d['ensemble_probability'].values()])
    keys = list(d['ensemble_probability'].keys())
    assert keys == [format(k, '0%db' % n) for k in range(1 << n)], 'unexpected key order'
    zi = z_sublattice(n)
    si = sample_indices(n, seed)
    meta = {'generator': 'tests/golden/make_c2_fixture.py', 'n': n, 'layers': layers, 'seed': seed,
            'options': opts, 'seconds': wall, 'cpu_count': os.cpu_count(),
            'clock_cycles': int(res['number_of_clock_cycles'])}
    out = os.path.join(HERE, 'c2_qft_n%d_L%d_s%d.npz' % (n, layers, seed))
    np.savez_compressed(out, probs=probs, z_idx=zi.astype(np.uint32), z_val=coeff[zi],
                        idx=si.astype(np.uint32), val=coeff[si],
                        coeff_sum=np.float64(coeff.sum()), coeff_abs_sum=np.float64(np.abs(coeff).sum()),
                        clock_cycles=np.int64(res['number_of_clock_cycles']),
                        meta=np.array(json.dumps(meta)))
    print('wrote %s: %d levels, %.0f s' % (out, res['number_of_clock_cycles'], wall))


if __name__ == '__main__':
    main()
