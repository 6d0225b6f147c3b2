"""The reference's own dm_simulator, loaded by oracle/refload.py, against the oracle.

oracle/_ref holds the reference's two hot-path files byte-compiled by
oracle/build_ref.py (run by build() where the reference tree exists); the
CPU legs of bench.py time that code.  Skipped where neither the tree nor the
byte code is present.
"""
import copy

import numpy as np
import pytest

import qiskit_aakash_gb300 as dmg
from oracle import dm_oracle as O
from oracle import refload


@pytest.fixture(scope='module')
def ref():
    if refload.available() is None:
        pytest.skip('reference dm_simulator not available (no tree, no oracle/_ref)')
    return refload.load()


@pytest.mark.parametrize('n,layers,seed', [(5, 3, 0), (6, 2, 1)])
def test_reference_matches_oracle(ref, n, layers, seed):
    qc = dmg.random_layer_circuit(n, layers, seed, barrier_after_gate=True)
    opts = dmg.noise_options(depolarisation=1e-3, decoherence=0.995, decay=0.998, rotation_sigma=1e-3)
    opts['compute_densitymatrix'] = False
    ref.DmSimulatorPy.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
    b = ref.DmSimulatorPy()
    b._set_options(qobj_config=None, backend_options=copy.deepcopy(opts))
    want = b.run_experiment(qc.to_experiment())
    got = O.OracleDmSimulator(copy.deepcopy(opts)).run_experiment(qc.to_experiment())
    assert want['number_of_clock_cycles'] == got['number_of_clock_cycles']
    np.testing.assert_allclose(np.asarray(got['data']['coeffmatrix']) * 2 ** n,
                               np.asarray(want['data']['coeffmatrix']) * 2 ** n, rtol=0, atol=1e-12)
    pw = np.array(list(want['data']['ensemble_probability'].values()), dtype=float)
    pg = np.array(list(got['data']['ensemble_probability'].values()), dtype=float)
    np.testing.assert_allclose(pg, pw, rtol=0, atol=1e-12)


def test_byte_code_is_the_python_version_of_this_interpreter():
    import importlib.util
    import os
    if not all(os.path.isfile(refload.pyc_path(m)) for m in refload.MODULES):
        pytest.skip('oracle/_ref not built')
    with open(refload.pyc_path('dm_simulator'), 'rb') as f:
        assert f.read(4) == importlib.util.MAGIC_NUMBER
