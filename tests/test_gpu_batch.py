"""Batched noise sweep on the GPU: every instance of one dm_batch_run launch
against the oracle (small instances) and against the single-experiment
backend (larger ones), graph replay, and table rejection on the host."""
import ctypes

import numpy as np
import pytest

from oracle import dm_oracle as O
from qiskit_aakash_gb300 import _native as N
from qiskit_aakash_gb300 import batch as B

pytestmark = pytest.mark.gpu

TOL = {'double': 1e-12, 'single': 1e-6}     # max-abs probability error, and probability L1
# Probability L1 of the batched tensor-core form: its FP16-split rounds keep the 1e-6 max-abs bound, but
# on low-noise instances (noise ~1e-4, large coefficients surviving every round) the L1 over 4,096
# outcomes of a 12-qubit instance reaches ~1.3e-6 (the CUDA-core FP32 form stays below 1e-6).
TC_BATCH_L1 = 5e-6


def oracle_probs(spec):
    exp, opts = B.instance_experiment(spec)
    res = O.OracleDmSimulator(dict(opts, compute_densitymatrix=False)).run_experiment(exp)
    p = res['data']['ensemble_probability']
    return np.array([p[k] for k in O.bitstring_keys(spec['n'])])


@pytest.fixture(scope='module')
def small_sweep():
    specs = B.sweep_specs(40, seed=21, n_range=(3, 8), depth_range=(2, 12))
    return specs, [oracle_probs(s) for s in specs]


@pytest.mark.parametrize('precision', ['double', 'single'])
def test_batch_matches_oracle(small_sweep, precision):
    specs, want = small_sweep
    prog = B.BatchProgram(B.BatchTables(specs, precision))
    prog.launch()
    got = prog.results()
    for i, spec in enumerate(specs):
        assert np.max(np.abs(got[i] - want[i])) < TOL[precision], (i, spec)
        assert np.abs(got[i] - want[i]).sum() < max(TOL[precision], 1e-12 * len(want[i])), (i, spec)
        assert abs(got[i].sum() - 1.0) < TOL[precision]


@pytest.mark.parametrize('precision,kmax', [('single', {8: 5, 7: 4, 6: 4}), ('double', {8: 4, 7: 4, 6: 5})])
def test_batch_resident_axes_do_not_change_results(small_sweep, precision, kmax):
    specs, want = small_sweep
    prog = B.BatchProgram(B.BatchTables(specs, precision, kmax=kmax))
    prog.launch()
    for i, g in enumerate(prog.results()):
        assert np.max(np.abs(g - want[i])) < TOL[precision]


def test_batch_large_instances_match_backend():
    from qiskit_aakash_gb300.dm_simulator import DmSimulatorGPU
    specs = B.sweep_specs(6, seed=4, n_range=(10, 12), depth_range=(8, 20))
    for precision in ('double', 'single'):
        prog = B.BatchProgram(B.BatchTables(specs, precision))
        prog.launch()
        got = prog.results()
        for i, spec in enumerate(specs):
            exp, opts = B.instance_experiment(spec)
            DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
            be = DmSimulatorGPU()
            be._set_options(backend_options=dict(opts, compute_densitymatrix=False, precision='double'))
            res = be.run_experiment(exp)
            p = res['data']['ensemble_probability']
            ref = np.array([p[k] for k in O.bitstring_keys(spec['n'])])
            assert np.max(np.abs(got[i] - ref)) < TOL[precision], (precision, i)
            assert np.abs(got[i] - ref).sum() < max(TOL[precision], 1e-12 * len(ref)), (precision, i)


def test_batch_graph_replay_and_rerun():
    import torch
    specs = B.sweep_specs(30, seed=8, n_range=(3, 9), depth_range=(2, 10))
    prog = B.BatchProgram(B.BatchTables(specs, 'single'))
    prog.capture()
    torch.cuda.synchronize()
    first = [r.copy() for r in prog.results()]
    prog.probs.zero_()
    prog.states.fill_(float('nan'))
    for _ in range(3):
        prog.run()
    torch.cuda.synchronize()
    for a, b in zip(first, prog.results()):
        assert np.array_equal(a, b)


def test_batch_rejects_bad_tables():
    specs = B.sweep_specs(3, seed=2, n_range=(4, 5), depth_range=(2, 4))
    prog = B.BatchProgram(B.BatchTables(specs, 'single'))
    t = prog.t
    bad = (N.DmBatchPass * t.npasses).from_buffer_copy(bytes(t.passes))
    bad[0].axes[0] -= 1
    vp = ctypes.c_void_p
    args = lambda insts, passes, npasses: (  # noqa: E731
        N.DM_F32, vp(prog.states.data_ptr()), ctypes.c_size_t(t.states_count), vp(prog.probs.data_ptr()),
        ctypes.c_size_t(t.probs_count), vp(prog.mats_dev.data_ptr()), ctypes.c_size_t(t.mats.size), insts,
        vp(prog.insts_dev.data_ptr()), t.ninst, passes, vp(prog.passes_dev.data_ptr()), npasses,
        vp(prog.counter.data_ptr()), vp(prog.status.data_ptr()), None)
    with pytest.raises(N.NativeError) as e:
        N.call('dm_batch_run', *args(t.insts, bad, t.npasses))
    assert e.value.code == N.DM_ERR_PROGRAM
    insts = (N.DmBatchInstance * t.ninst).from_buffer_copy(bytes(t.insts))
    insts[0].state_off = t.states_count
    with pytest.raises(N.NativeError) as e:
        N.call('dm_batch_run', *args(insts, t.passes, t.npasses))
    assert e.value.code == N.DM_ERR_ARG
    insts = (N.DmBatchInstance * t.ninst).from_buffer_copy(bytes(t.insts))
    insts[0].n = 13
    with pytest.raises(N.NativeError) as e:
        N.call('dm_batch_run', *args(insts, t.passes, t.npasses))
    assert e.value.code == N.DM_ERR_RANGE
    insts = (N.DmBatchInstance * t.ninst).from_buffer_copy(bytes(t.insts))
    insts[0].mats_len = 1
    with pytest.raises(N.NativeError):
        N.call('dm_batch_run', *args(insts, t.passes, t.npasses))


TC_KMAX = {n: B.TC for n in range(7, 13)}


def test_tensor_core_batch_matches_oracle(small_sweep):
    """Mixed batch: 7- and 8-qubit instances on the tensor cores, the rest on the CUDA-core rounds."""
    specs, want = small_sweep
    T = B.BatchTables(specs, 'single', kmax=TC_KMAX)
    assert T.tc.ninst > 0 and T.ninst > 0
    prog = B.BatchProgram(T)
    prog.launch()
    got = prog.results()
    for i, spec in enumerate(specs):
        assert np.max(np.abs(got[i] - want[i])) < TOL['single'], (i, spec)
        assert np.abs(got[i] - want[i]).sum() < TOL['single'], (i, spec)
        assert abs(got[i].sum() - 1.0) < TOL['single']


def test_tensor_core_batch_large_instances_match_fp64_backend():
    from qiskit_aakash_gb300.dm_simulator import DmSimulatorGPU
    specs = B.sweep_specs(8, seed=14, n_range=(9, 12), depth_range=(6, 24))
    T = B.BatchTables(specs, 'single', kmax=TC_KMAX)
    assert T.tc.ninst == len(specs)
    prog = B.BatchProgram(T)
    prog.launch()
    got = prog.results()
    for i, spec in enumerate(specs):
        exp, opts = B.instance_experiment(spec)
        DmSimulatorGPU.DEFAULT_OPTIONS['rotation_error'] = {'rx': [1., 0.], 'ry': [1., 0.], 'rz': [1., 0.]}
        be = DmSimulatorGPU()
        be._set_options(backend_options=dict(opts, compute_densitymatrix=False, precision='double'))
        res = be.run_experiment(exp)
        p = res['data']['ensemble_probability']
        ref = np.array([p[k] for k in O.bitstring_keys(spec['n'])])
        assert np.max(np.abs(got[i] - ref)) < TOL['single'], i
        assert np.abs(got[i] - ref).sum() < TC_BATCH_L1, i


def test_tensor_core_batch_graph_replay():
    import torch
    specs = B.sweep_specs(20, seed=9, n_range=(6, 10), depth_range=(2, 8))
    prog = B.BatchProgram(B.BatchTables(specs, 'single', kmax=TC_KMAX))
    prog.capture()
    torch.cuda.synchronize()
    first = [r.copy() for r in prog.results()]
    prog.probs.zero_()
    prog.states.fill_(float('nan'))
    for _ in range(3):
        prog.run()
    torch.cuda.synchronize()
    for a, b in zip(first, prog.results()):
        assert np.array_equal(a, b)


def test_tensor_core_batch_rejects_bad_tables():
    specs = B.sweep_specs(2, seed=2, n_range=(7, 8), depth_range=(2, 4))
    prog = B.BatchProgram(B.BatchTables(specs, 'single', kmax=TC_KMAX))
    tc = prog.t.tc
    t = prog.t
    vp = ctypes.c_void_p

    def call(insts, passes):
        N.call('dm_batch_run_tc', vp(prog.states.data_ptr()), ctypes.c_size_t(t.states_count),
               vp(prog.probs.data_ptr()), ctypes.c_size_t(t.probs_count), vp(prog.tc_mats_dev.data_ptr()),
               ctypes.c_size_t(tc.mats.size), insts, vp(prog.tc_insts_dev.data_ptr()), tc.ninst, passes,
               vp(prog.tc_passes_dev.data_ptr()), tc.npasses, vp(prog.counter.data_ptr()),
               vp(prog.tc_scratch.data_ptr()), ctypes.c_size_t(prog.tc_scratch.numel()),
               vp(prog.status.data_ptr()), None)

    def fresh_passes():
        return (N.DmBatchTcPass * tc.npasses).from_buffer_copy(bytes(tc.passes))

    bad = fresh_passes()
    bad[0].tables.rounds[0].digits[0] = (bad[0].ops.round_axes[0][0] + 1) % 7   # table and op digits disagree
    with pytest.raises(N.NativeError) as e:
        call(tc.insts, bad)
    assert e.value.code == N.DM_ERR_PROGRAM
    bad = fresh_passes()
    bad[0].ops.k = 6
    with pytest.raises(N.NativeError) as e:
        call(tc.insts, bad)
    assert e.value.code == N.DM_ERR_PROGRAM
    bad = fresh_passes()
    bad[0].tables.rounds[0].rowc[0] = 0                                  # a zero destination offset
    with pytest.raises(N.NativeError) as e:
        call(tc.insts, bad)
    assert e.value.code == N.DM_ERR_PROGRAM
    insts = (N.DmBatchInstance * tc.ninst).from_buffer_copy(bytes(tc.insts))
    insts[0].n = 6
    with pytest.raises(N.NativeError) as e:
        call(insts, tc.passes)
    assert e.value.code == N.DM_ERR_RANGE
    with pytest.raises(N.NativeError) as e:
        N.call('dm_batch_run_tc', vp(prog.states.data_ptr()), ctypes.c_size_t(t.states_count),
               vp(prog.probs.data_ptr()), ctypes.c_size_t(t.probs_count), vp(prog.tc_mats_dev.data_ptr()),
               ctypes.c_size_t(tc.mats.size), tc.insts, vp(prog.tc_insts_dev.data_ptr()), tc.ninst, tc.passes,
               vp(prog.tc_passes_dev.data_ptr()), tc.npasses, vp(prog.counter.data_ptr()),
               vp(prog.tc_scratch.data_ptr()), ctypes.c_size_t(16), vp(prog.status.data_ptr()), None)
    assert e.value.code == N.DM_ERR_ARG
    prog.launch()                                       # the good tables still run
    assert int(prog.status.item()) == 0
