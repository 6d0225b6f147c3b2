"""``DmSimulatorGPU``: the reference's ``dm_simulator`` backend on a GB300.

Same contract as ``DmSimulatorPy`` (qiskit/providers/basicaer/
dm_simulator.py:61-1313): configuration and option names, ``run`` /
``_run_job`` / ``run_experiment``, the per-level semantics (merge, levels,
memory noise after every level), the measurement family and the result
dictionary.  The difference is where the state lives: a device-resident
vector of 4**n Pauli coefficients updated by the sm_103a kernels of
libdmgb300.so, with the operations of consecutive levels fused into
shared-memory tile passes.

Behaviour kept from the reference on purpose (its users see it):
* ``rotation_error`` updates the class-level default dict in place
  (dm_simulator.py:182, :212-213), so values persist into later runs;
* ``bell_depolarization_factor`` is stored on an attribute the Bell
  measurement never reads (:240): Bell measurements use 1.0;
* ``depolarization_factor`` acts only at measurement (:281, :1082-1133);
* memory noise runs once per level on every qubit, idle or not (:1173-1177);
* single-basis measurements update the state but record no classical bits;
* the Bell measurement addresses qubits n-1-q (the reversed reshape of :741);
* among several single measurements in one level the one after each applied
  measurement is skipped (the list is modified while iterated, :1100).
Differences (the reference fails on these inputs):
* conditional gates driven by ``bfunc`` raise ``BasicAerError`` up front
  (the reference's levelling raises AttributeError on bfunc, which has no
  qubits: basicaertools.py:549);
* plain-string measurement parameters are treated like sympy Symbols;
* the initial-state checks raise ``InitialStateError`` (a BasicAerError and
  an AttributeError) with a readable message.
GB300 options (absent from the reference): ``precision`` ('double', the
default and the parity form, or 'single'), ``fusion`` (fused tile passes,
default True), ``tile_axes`` (resident axes per tile), ``register_rounds``
(apply a pass's operations in register rounds, default True), ``tensor_cores``
(FP32 passes on tcgen05 as 64x64 transfer matrices in a 3-way FP16 split, default True), ``tma``
(tensor-core passes with TMA-fed tiles where a pass fits them, default True),
``compose`` ('device', the default: each tensor-core round's 64x64 matrix is
composed in FP64 on the GPU from the operations' coefficients; 'host': in
numpy, with the FP16 images uploaded) and
``coefficients_to_host`` (default True; False leaves ``coeffmatrix`` /
``densitymatrix`` out of the result, for callers that only need the
measurement data of a large register) and ``counts_shots`` / ``counts_seed``
(default 0: off; with shots > 0 every ensemble measurement also reports
``counts``, {bit string: count} of that many shots drawn on the device from
its outcome probabilities; the reference reports probabilities only) and
``fp64_check`` (default False; with precision 'single' the experiment is run
a second time in FP64 on the device and the result's data gains
``max_abs_coeff_err`` (max |2**n (a32 - a64)| over the final state),
``prob_l1_err`` (the largest L1 distance of its probability outputs) and
``trace_err``).  Every run ends with a trace-preservation check: 2**n a_0,
read from the device in FP64, must be 1 within TRACE_TOL of the precision,
else BasicAerError (the reference checks a_0 = 2**-n on the initial state
only, dm_simulator.py:363).
"""
import copy
import logging
import time
import uuid
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import _native as N
from . import program as P
from .engine import DeviceState
from .exceptions import BasicAerError, InitialStateError, QiskitError
from .scheduler import levelize, merge_single_gates

logger = logging.getLogger(__name__)

try:  # pragma: no cover - only where qiskit-aakash is installed
    from qiskit.providers import BaseBackend as _Base
    from qiskit.providers.models import QasmBackendConfiguration as _Config
except Exception:  # noqa: BLE001
    class _Config:
        """Attribute view of a backend configuration dict."""

        def __init__(self, **kw):
            self.__dict__.update(kw)

        @classmethod
        def from_dict(cls, d):
            return cls(**copy.deepcopy(d))

        def to_dict(self):
            return copy.deepcopy(self.__dict__)

    class _Base:
        def __init__(self, configuration, provider=None):
            self._configuration = configuration
            self._provider = provider

        def configuration(self):
            return self._configuration

        def name(self):
            return self._configuration.backend_name

        def provider(self):
            return self._provider

        def status(self):
            return {'backend_name': self.name(), 'operational': True, 'pending_jobs': 0}

        def __repr__(self):
            return "<%s('%s')>" % (type(self).__name__, self.name())


class DmGpuJob:
    """Job handle with BasicAerJob's interface (basicaerjob.py:44-138).

    The reference runs jobs in a forked process pool (basicaerjob.py:51-54);
    a CUDA context does not survive fork, so this job runs in a worker thread
    of the calling process.
    """

    _executor = ThreadPoolExecutor(max_workers=1, thread_name_prefix='dm_gb300')

    def __init__(self, backend, job_id, fn, qobj):
        self._backend = backend
        self._job_id = job_id
        self._fn = fn
        self._qobj = qobj
        self._future = None

    def submit(self):
        if self._future is not None:
            raise BasicAerError('We have already submitted the job!')
        self._future = self._executor.submit(self._fn, self._job_id, self._qobj)

    def result(self, timeout=None):
        if self._future is None:
            raise BasicAerError('Job not submitted yet!')
        return self._future.result(timeout=timeout)

    def cancel(self):
        return self._future.cancel() if self._future else False

    def status(self):
        if self._future is None:
            return 'INITIALIZING'
        if self._future.running():
            return 'RUNNING'
        if self._future.cancelled():
            return 'CANCELLED'
        if self._future.done():
            return 'ERROR' if self._future.exception() is not None else 'DONE'
        return 'QUEUED'

    def backend(self):
        return self._backend

    def qobj(self):
        return self._qobj

    def job_id(self):
        return self._job_id


_PAULI = {'I': 0, 'X': 1, 'Y': 2, 'Z': 3}
_AXIS = {'X': 1, 'Y': 2, 'Z': 3}


class DmSimulatorGPU(_Base):
    """Pauli-basis density-matrix simulator on one GB300 (drop-in for DmSimulatorPy)."""

    MAX_QUBITS_MEMORY = N.DM_MAX_QUBITS

    DEFAULT_CONFIGURATION = {
        'backend_name': 'dm_simulator',
        'backend_version': '2.0.0',
        'n_qubits': MAX_QUBITS_MEMORY,
        'url': 'https://github.com/Qiskit/qiskit-terra',
        'simulator': True,
        'local': True,
        'conditional': True,
        'open_pulse': False,
        'memory': True,
        'max_shots': 1,
        'coupling_map': None,
        'description': 'A GB300 density matrix simulator for qasm experiments (Pauli basis)',
        'basis_gates': ['u1', 'u2', 'u3', 'cx', 'id', 'unitary'],
        'gates': [
            {'name': 'u1', 'parameters': ['lambda'], 'qasm_def': 'gate u1(lambda) q { U(0,0,lambda) q; }'},
            {'name': 'u2', 'parameters': ['phi', 'lambda'],
             'qasm_def': 'gate u2(phi,lambda) q { U(pi/2,phi,lambda) q; }'},
            {'name': 'u3', 'parameters': ['theta', 'phi', 'lambda'],
             'qasm_def': 'gate u3(theta,phi,lambda) q { U(theta,phi,lambda) q; }'},
            {'name': 'cx', 'parameters': ['c', 't'], 'qasm_def': 'gate cx c,t { CX c,t; }'},
            {'name': 'id', 'parameters': ['a'], 'qasm_def': 'gate id a { U(0,0,0) a; }'},
            {'name': 'unitary', 'parameters': ['matrix'], 'qasm_def': 'unitary(matrix) q1, q2,...'},
        ],
    }

    DEFAULT_OPTIONS = {
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

    SHOW_FINAL_STATE = True
    PLOTTING = False
    SHOW_PARTITION = False
    DEBUG = True
    STORE_LOCAL = False
    COMPARE = False
    FILE_EXIST = False
    MERGE = True

    def __init__(self, configuration=None, provider=None):
        super().__init__(configuration=(configuration or _Config.from_dict(self.DEFAULT_CONFIGURATION)),
                         provider=provider)
        self._classical_memory = 0
        self._classical_register = 0
        self._dev = None
        self._number_of_cmembits = 0
        self._number_of_qubits = 0
        self._custom_densitymatrix = None
        self._initial_densitymatrix = self.DEFAULT_OPTIONS["initial_densitymatrix"]
        self._chop_threshold = self.DEFAULT_OPTIONS["chop_threshold"]
        self._qobj_config = None
        self._error_params = {}
        self._rotation_error = None
        self._tsp_model_error = None
        self._thermal_factor = None
        self._decoherence_factor = None
        self._decay_factor = None
        self._depolarization_factor = None
        self._bell_depolarization_factor = None
        self._get_den_mat = True
        self._fidelity = None
        self._density_matrix_stored = None
        # GB300 options (not in the reference)
        self._precision = 'double'
        self._fusion = True
        self._tile_axes = None
        self._coefficients_to_host = True
        self._counts_shots = 0
        self._counts_seed = 0
        self._register_rounds = True
        self._tensor_cores = True
        self._tma = True
        self._compose = 'device'
        self._fp64_check = False
        self.last_run_stats = {}
        self._record_next = False
        self.recorded_state = None
        self._state_factory = DeviceState

    def record_experiment(self, experiment):
        """Run one experiment and keep its device state with a replayable call tape.

        ``self.recorded_state.replay()`` then re-issues the experiment's device
        work (state set-up, fused passes, measurement read-outs into the same
        device buffers) with no host-side planning or transfers; used to time
        the device path with its inputs resident.
        """
        self._record_next = True
        try:
            return self.run_experiment(experiment)
        finally:
            self._record_next = False

    def compile_experiment(self, experiment):
        """Run one experiment's host logic against a recorder instead of a device state.

        Returns the recorder (``batch.HostRecorder``) holding the initial
        product state, the op stream (merged gates, levelled noise,
        measurement updates) and the read-outs the experiment asks for; the
        batched sweep runner executes such streams for many instances in
        one launch.  Read-out values seen by the host logic are zeros.
        """
        from .batch import HostRecorder
        holder = {}

        def keep(n, **kw):
            holder['rec'] = HostRecorder(n, **kw)
            return holder['rec']

        self._state_factory = keep
        try:
            self.run_experiment(experiment)
        finally:
            self._state_factory = DeviceState
        return holder['rec']

    # ------------------------------------------------------------------ options
    def _set_options(self, qobj_config=None, backend_options=None):
        """dm_simulator.py:177-271, plus 'precision', 'fusion', 'tile_axes'."""
        self._initial_densitymatrix = self.DEFAULT_OPTIONS["initial_densitymatrix"]
        self._chop_threshold = self.DEFAULT_OPTIONS["chop_threshold"]
        self._rotation_error = self.DEFAULT_OPTIONS["rotation_error"]
        self._tsp_model_error = self.DEFAULT_OPTIONS["tsp_model_error"]
        self._thermal_factor = self.DEFAULT_OPTIONS["thermal_factor"]
        self._decoherence_factor = self.DEFAULT_OPTIONS["decoherence_factor"]
        self._decay_factor = self.DEFAULT_OPTIONS["decay_factor"]
        self._depolarization_factor = self.DEFAULT_OPTIONS["depolarization_factor"]
        self._bell_depolarization_factor = self.DEFAULT_OPTIONS["bell_depolarization_factor"]
        self._counts_shots = 0          # shot counts are a per-run request
        self._counts_seed = 0
        if backend_options is None:
            backend_options = {}
        if 'initial_densitymatrix' in backend_options:
            self._initial_densitymatrix = backend_options['initial_densitymatrix']
        elif hasattr(qobj_config, 'initial_densitymatrix'):
            self._initial_densitymatrix = qobj_config.initial_densitymatrix
        if 'custom_densitymatrix' in backend_options:
            self._custom_densitymatrix = backend_options['custom_densitymatrix']
        if 'rotation_error' in backend_options:
            re = backend_options['rotation_error']
            if type(re) != dict or not all(x in ['rx', 'ry', 'rz'] for x in re):  # noqa: E721
                raise BasicAerError('Error! Incorrect Rotation Error parameters, Expected argument : A dict '
                                    'with rotation gate as key and a list of 2 reals ranging between 0 and 1 '
                                    'both inclusive as their values.')
            for gt, vl in re.items():
                self._rotation_error.update({gt: vl})
        if 'tsp_model_error' in backend_options:
            t = backend_options['tsp_model_error']
            if type(t) != list or len(t) != 2 or t[0] > 1 or t[1] > 1:  # noqa: E721
                raise BasicAerError('Error! Incorrect transition model error parameter, Expected argument : '
                                    'A list of 2 reals ranging between 0 and 1 both inclusive.')
            self._tsp_model_error = t
        if 'thermal_factor' in backend_options:
            self._thermal_factor = backend_options['thermal_factor']
        if 'decoherence_factor' in backend_options:
            self._decoherence_factor = backend_options['decoherence_factor']
        if 'decay_factor' in backend_options:
            self._decay_factor = backend_options['decay_factor']
        if 'depolarization_factor' in backend_options:
            self._depolarization_factor = backend_options['depolarization_factor']
        if 'bell_depolarization_factor' in backend_options:
            self.bell_depolarization_factor = backend_options['bell_depolarization_factor']
        if 'chop_threshold' in backend_options:
            self._chop_threshold = backend_options['chop_threshold']
        elif hasattr(qobj_config, 'chop_threshold'):
            self._chop_threshold = qobj_config.chop_threshold
        if 'compute_densitymatrix' in backend_options:
            self._get_den_mat = backend_options['compute_densitymatrix']
        if 'merge' in backend_options:
            self.MERGE = backend_options['merge']
        if 'plot' in backend_options:
            self.PLOTTING = backend_options['plot']
        if 'show_partition' in backend_options:
            self.SHOW_PARTITION = backend_options['show_partition']
        if 'store_densitymatrix' in backend_options:
            self.STORE_LOCAL = backend_options['store_densitymatrix']
        if 'compare' in backend_options:
            self.COMPARE = backend_options['compare']
            try:
                self._density_matrix_stored = np.load('stored_coefficients.npy')
                self.FILE_EXIST = True
            except FileNotFoundError:
                print('Stored Coefficient File does not exist')
        if 'precision' in backend_options:
            if backend_options['precision'] not in ('double', 'single'):
                raise BasicAerError("precision must be 'double' or 'single'")
            self._precision = backend_options['precision']
        if 'fusion' in backend_options:
            self._fusion = bool(backend_options['fusion'])
        if 'tile_axes' in backend_options:
            self._tile_axes = int(backend_options['tile_axes'])
        if 'tensor_cores' in backend_options:
            self._tensor_cores = bool(backend_options['tensor_cores'])
        if 'tma' in backend_options:
            self._tma = bool(backend_options['tma'])
        if 'compose' in backend_options:
            if backend_options['compose'] not in ('device', 'host'):
                raise BasicAerError("compose must be 'device' or 'host'")
            self._compose = backend_options['compose']
        if 'register_rounds' in backend_options:
            self._register_rounds = bool(backend_options['register_rounds'])
        if 'coefficients_to_host' in backend_options:
            self._coefficients_to_host = bool(backend_options['coefficients_to_host'])
        if 'counts_shots' in backend_options:
            shots = int(backend_options['counts_shots'])
            if shots < 0:
                raise BasicAerError('counts_shots must be >= 0')
            self._counts_shots = shots
        if 'counts_seed' in backend_options:
            self._counts_seed = int(backend_options['counts_seed'])
        if 'fp64_check' in backend_options:
            self._fp64_check = bool(backend_options['fp64_check'])

    def _initialize_errors(self):
        """dm_simulator.py:273-282."""
        self._error_params.update({'one_qubit_gates': self._rotation_error})
        self._error_params.update({'two_qubit_gates': self._tsp_model_error})
        self._error_params.update({'memory': {'thermalization': self._thermal_factor,
                                              'decoherence': self._decoherence_factor,
                                              'amplitude_decay': self._decay_factor}})
        self._error_params.update({'measurement': self._depolarization_factor,
                                   'measurement_bell': self._bell_depolarization_factor})

    # ------------------------------------------------------------------- state
    def _initialize_densitymatrix(self):
        """dm_simulator.py:284-349: product states built on the device."""
        n = self._number_of_qubits
        dev = self._dev
        if self._initial_densitymatrix is None:
            per = {None: [1, 0, 0, 1], 'max_mixed': [1, 0, 0, 0], 'uniform_superpos': [1, 1, 0, 0],
                   'thermal_state': [1, 0, 0, 2 * self._thermal_factor - 1]}
            if self._custom_densitymatrix not in per:
                raise BasicAerError('_custom_densitymatrix value is invalid')
            dev.init_product([per[self._custom_densitymatrix]] * n, 0.5 ** n)
        elif self._custom_densitymatrix == 'binary_string':
            bits = self._initial_densitymatrix
            if len(bits) != n:
                raise BasicAerError('Wrong input binary string length')
            # the string's first character ends up on the fastest axis (qubit n-1)
            vecs = [[1, 0, 0, 1 if ch == '0' else -1] for ch in reversed(bits)]
            dev.init_product(vecs, 0.5 ** n)
        elif self._custom_densitymatrix == 'stored_density_matrix':
            try:
                st = np.load('stored_density_matrix.npy')
            except FileNotFoundError:
                print('Stored Coefficient File does not exist')
                raise BasicAerError('stored_density_matrix.npy not found')
            if len(st) != 4 ** n:
                raise BasicAerError('Wrong input stored density matrix')
            dev.load(st)
        else:
            raise BasicAerError('_custom_densitymatrix value is invalid')

    def _validate_initial_densitymatrix(self):
        """dm_simulator.py:351-365: the trace coefficient must be 2**-n."""
        if self._initial_densitymatrix is None:
            return
        n = self._number_of_qubits
        a0 = self._dev.gather([0])[0]
        if a0 != 2.0 ** (-n):
            raise InitialStateError('Trace of initial densitymatrix is not one: {} != {}'.format(a0 * 2 ** n, 1))

    # ------------------------------------------------------------- operations
    def _add_unitary_single(self, gate, qubit):
        """dm_simulator.py:367-384: the u1/u3 rotations as one composed 4x4 map."""
        m = P.rotations_ptm(gate, self._error_params['one_qubit_gates'])
        self._dev.map1(qubit, m, tag=('rot', tuple((axis, float(angle)) for axis, angle in gate)))

    def _add_unitary_two(self, qubit0, qubit1):
        """dm_simulator.py:386-395 (cx_gate_dm_matrix, basicaertools.py:310-392)."""
        n = self._number_of_qubits
        if qubit0 == qubit1 or qubit0 >= n or qubit1 >= n:
            raise QiskitError('Qubit Labels out of bound in CX Gate')
        self._dev.cx(qubit0, qubit1, self._error_params['two_qubit_gates'])

    def _add_decoherence_and_amp_decay(self, level, f, p, g):
        """dm_simulator.py:397-425: memory noise on every qubit."""
        key = (f, p, g)
        cached = getattr(self, '_noise_map', None)
        if cached is None or cached[0] != key:     # the same map every level of a run
            m = P.noise_ptm(f, p, g)
            cached = self._noise_map = (key, m, np.array_equal(m, P.IDENTITY4))
        if cached[2]:
            return
        m = cached[1]
        for q in range(self._number_of_qubits):
            self._dev.map1(q, m, tag=('noise',))

    def _add_qasm_measure(self, basis, qubit, err_param, nvec=None):
        self._dev.map1(qubit, P.measure_ptm(basis, err_param, nvec))

    def _add_qasm_measure_X(self, qubit, cmembit, cregbit=None, err_param=1.0):
        """dm_simulator.py:574-602 (the returned probability is not used by the reference)."""
        self._add_qasm_measure('X', qubit, err_param)

    def _add_qasm_measure_Y(self, qubit, cmembit, cregbit=None, err_param=1.0):
        """dm_simulator.py:604-632."""
        self._add_qasm_measure('Y', qubit, err_param)

    def _add_qasm_measure_Z(self, qubit, cmembit, cregbit=None, err_param=1.0):
        """dm_simulator.py:634-664."""
        self._add_qasm_measure('Z', qubit, err_param)

    def _add_qasm_measure_N(self, qubit, cmembit, cregbit=None, n=np.array([0.0, 0.0, 1.0]), err_param=1.0):
        """dm_simulator.py:666-704."""
        self._add_qasm_measure('N', qubit, err_param, n)

    def _unit_vector_normalisation(self, n):
        """dm_simulator.py:706-719."""
        n = np.asarray(n, dtype=float)
        norm = np.linalg.norm(n)
        if norm == 1:
            return n
        logger.warning('Given direction for the measurement was not normalised. '
                       'It has been normalised to be unit vector!!')
        return n / norm

    def _add_qasm_reset(self, qubit):
        """dm_simulator.py:810-823."""
        self._dev.map1(qubit, P.reset_ptm())

    def _add_ensemble_measure(self, basis, add_param, err_param):
        """dm_simulator.py:427-481: probabilities of all 2**n outcomes (state unchanged)."""
        n = self._number_of_qubits
        if basis == 'N':
            probs = self._dev.nbasis_probs(np.asarray(add_param, dtype=float), err_param)
        elif basis in _AXIS:
            probs = self._dev.axis_probs([_AXIS[basis]] * n, err_param)
        else:
            raise KeyError(basis)
        prob = dict(zip(_bit_keys(n), probs))
        max_str = max(prob, key=prob.get)
        max_prob = prob[max_str]
        if self.STORE_LOCAL:
            self._store_density_matrix()
        if self.COMPARE and self.FILE_EXIST:
            self._fidelity = self._state_overlap(self._density_matrix_stored, None)
        return prob, max_str, max_prob

    def _add_partial_measure(self, measured_qubits, cmembits, cregbits, err_param, basis, add_param=None):
        """dm_simulator.py:492-538: probabilities of the measured qubits, then their state updates."""
        n = self._number_of_qubits
        m = len(measured_qubits)
        if basis == 'N':
            full, _, _ = self._add_ensemble_measure(basis, add_param, err_param)
            arr = np.array(list(full.values()))
            others = tuple(sorted(set(range(n)) - set(measured_qubits)))
            probs = np.reshape(np.sum(np.reshape(arr, [2] * n), axis=others), 2 ** m)
        else:
            mode = [_AXIS[basis] if q in set(measured_qubits) else 0 for q in range(n)]
            probs = self._dev.axis_probs(mode, err_param)
            if self.STORE_LOCAL:
                self._store_density_matrix()
            if self.COMPARE and self.FILE_EXIST:
                self._fidelity = self._state_overlap(self._density_matrix_stored, None)
        partial = dict(zip(_bit_keys(m), probs))
        max_str = max(partial, key=partial.get)
        max_prob = partial[max_str]
        for mqb, mcb, mcregb in list(zip(measured_qubits, cmembits, cregbits)):
            if basis == 'N' and add_param is not None:
                self._add_qasm_measure_N(mqb, mcb, mcregb, add_param, self._error_params['measurement'])
            else:
                self._add_qasm_measure(basis, mqb, self._error_params['measurement'])
        return partial, max_str, max_prob

    def _pauli_string_expectation(self, basis, err_param, add_param=None):
        """dm_simulator.py:540-572: project each qubit, then read one coefficient."""
        n = self._number_of_qubits
        for i in range(n):
            if basis[i] in _AXIS:
                self._add_qasm_measure(basis[i], i, err_param)
        idx = sum(_PAULI[c] * 4 ** (n - 1 - q) for q, c in enumerate(basis))
        if len(basis) != n:
            raise IndexError('too many indices for array')
        return self._dev.gather([idx])[0] * 2 ** n

    def _add_bell_basis_measure(self, qubit_1, qubit_2, err_param):
        """dm_simulator.py:721-777 (axes n-1-q as in the reference's reversed reshape)."""
        n = self._number_of_qubits
        q1, q2 = min(qubit_1, qubit_2), max(qubit_1, qubit_2)
        if q1 == q2 or q2 >= n or q1 < 0:
            raise ValueError('cannot reshape array for a Bell measurement on qubits %d, %d' % (qubit_1, qubit_2))
        A, B = n - 1 - q2, n - 1 - q1       # slower / faster axis in qubit terms
        sa, sb = 4 ** (n - 1 - A), 4 ** (n - 1 - B)
        idx = [i * sa + j * sb for i in range(4) for j in range(4)]
        red = np.reshape(self._dev.gather(idx), (4, 4)) * 2 ** (n - 2)
        self._dev.diag2(A, B, P.bell_projection_diag(err_param))
        k = self._dev.gather([i * sa + i * sb for i in range(4)]) * 2 ** n
        bp = [0.25 * (k[0] + k[1] - k[2] + k[3]), 0.25 * (k[0] - k[1] + k[2] + k[3]),
              0.25 * (k[0] + k[1] + k[2] - k[3]), 0.25 * (k[0] - k[1] - k[2] - k[3])]
        return dict(zip(['Bell_1', 'Bell_2', 'Bell_3', 'Bell_4'], bp)), red

    # ------------------------------------------------------------------- jobs
    def _validate(self, qobj):
        """dm_simulator.py:875-887."""
        n_qubits = qobj.config.n_qubits
        max_qubits = self.configuration().n_qubits
        if n_qubits > max_qubits:
            raise BasicAerError('Number of qubits {} '.format(n_qubits) +
                                'is greater than maximum ({}) '.format(max_qubits) +
                                'for "{}".'.format(self.name()))
        for experiment in qobj.experiments:
            name = experiment.header.name
            if 'measure' not in [op.name for op in experiment.instructions]:
                logger.warning('No measurements in circuit "%s", '
                               'classical register will remain all zeros.', name)

    def run(self, qobj, backend_options=None):
        """dm_simulator.py:889-919: set options, submit a job, return it."""
        self._set_options(qobj_config=qobj.config, backend_options=backend_options)
        job_id = str(uuid.uuid4())
        job = DmGpuJob(self, job_id, self._run_job, qobj)
        job.submit()
        return job

    def _run_job(self, job_id, qobj):
        """dm_simulator.py:921-948."""
        self._validate(qobj)
        result_list = []
        self._qobj_config = qobj.config
        start = time.time()
        for experiment in qobj.experiments:
            result_list.append(self.run_experiment(experiment))
        end = time.time()
        return {'backend_name': self.name(),
                'backend_version': self._configuration.backend_version,
                'qobj_id': qobj.qobj_id,
                'job_id': job_id,
                'results': result_list,
                'status': 'COMPLETED',
                'success': True,
                'time_taken': end - start,
                'header': qobj.header.as_dict()}

    def run_experiment(self, experiment):
        """dm_simulator.py:950-1196: one experiment, same result dictionary."""
        start_processing = time.time()
        n = experiment.config.n_qubits
        self._number_of_qubits = n
        self._number_of_cmembits = experiment.config.memory_slots
        self._classical_memory = 0
        self._classical_register = 0
        data = {}
        shadow_exp = copy.deepcopy(experiment) if self._fp64_check and self._precision == 'single' else None
        if any(op.name == 'bfunc' for op in experiment.instructions):
            raise BasicAerError('dm_simulator does not support conditional (bfunc) operations')
        self._dev = self._state_factory(n, precision=self._precision, fusion=self._fusion,
                                        tile_axes=self._tile_axes, rounds=self._register_rounds,
                                        tensor_cores=self._tensor_cores, tma=self._tma,
                                        compose=self._compose)
        if self._record_next:
            self._dev.record()
        launches0 = N.lib().dm_kernel_launch_count()
        self._initialize_densitymatrix()
        self._validate_initial_densitymatrix()
        self._initialize_errors()
        experiment.instructions = merge_single_gates(experiment.instructions, n, self.MERGE)
        partitioned_instructions, levels = levelize(experiment.instructions, n)
        if self.SHOW_PARTITION:
            self._describe_partition(partitioned_instructions)
        end_processing = time.time()
        start_runtime = time.time()
        part_measure = False
        mem = self._error_params['memory']
        for clock in range(levels):
            level = partitioned_instructions[clock]
            # same-basis partial measurement? (dm_simulator.py:1006-1018)
            for operation in level:
                if operation.name == 'measure':
                    basis = str(getattr(level[0], 'params', ['Z'])[0])
                    params = getattr(operation, 'params', ['Z'])
                    if str(params[0]) in ['X', 'Y', 'Z', 'N']:
                        if str(params[0]) == basis:
                            part_measure = True
                        else:
                            part_measure = False
                            break
                    else:
                        part_measure = False
                        continue
            # dm_simulator.py:1020-1170.  Single measurements remove themselves
            # from the level while it is iterated, as in the reference.
            for operation in level:
                conditional = getattr(operation, 'conditional', None)
                if isinstance(conditional, int):
                    if not (self._classical_register >> conditional) & 1:
                        continue
                elif conditional is not None:
                    mask = int(operation.conditional.mask, 16)
                    if mask > 0:
                        value = self._classical_memory & mask
                        while (mask & 0x1) == 0:
                            mask >>= 1
                            value >>= 1
                        if value != int(operation.conditional.val, 16):
                            continue
                name = operation.name
                if name in ('u1', 'u3'):
                    gate = _u_decomposition(name, operation.params)
                    self._add_unitary_single(gate, operation.qubits[0])
                elif name == 'cx':
                    self._add_unitary_two(operation.qubits[0], operation.qubits[1])
                elif name == 'reset':
                    self._add_qasm_reset(operation.qubits[0])
                elif name == 'barrier':
                    pass
                elif name == 'measure':
                    params = getattr(operation, 'params', ['Z'])
                    qubit = operation.qubits[0]
                    cmembit = operation.memory[0]
                    cregbit = operation.register[0] if hasattr(operation, 'register') else None
                    kind = str(params[0])
                    sngl = exp_m = ensm = False
                    if kind == 'Ensemble':
                        ensm = True
                    elif kind == 'Expect':
                        exp_m = True
                    elif len(level) == 1 or part_measure is not True:
                        sngl = True
                    if len(params) == 1:
                        params.append(None)
                    err = self._error_params['measurement']
                    if sngl:
                        if kind == 'X':
                            self._add_qasm_measure_X(qubit, cmembit, cregbit, err)
                        elif kind == 'Y':
                            self._add_qasm_measure_Y(qubit, cmembit, cregbit, err)
                        elif kind == 'N':
                            params[1] = self._unit_vector_normalisation(params[1])
                            self._add_qasm_measure_N(qubit, cmembit, cregbit, params[1], err)
                        elif kind == 'Bell':
                            pair = str(params[1])
                            bp, red = self._add_bell_basis_measure(
                                int(pair[0]), int(pair[1]), err_param=self._error_params['measurement_bell'])
                            data['bell_probabilities%s%s' % (pair[0], pair[1])] = bp
                            data['reduced_bell_densitymatrix%s%s' % (pair[0], pair[1])] = red
                        else:
                            self._add_qasm_measure_Z(qubit, cmembit, cregbit, err)
                        level.remove(operation)
                    elif part_measure:
                        qubits = [x.qubits[0] for x in level]
                        cmems = [x.memory[0] for x in level]
                        cregs = [x.register[0] if hasattr(x, 'register') else None for x in level]
                        add_param = params[1] if kind == 'N' else None
                        data['partial_probability'], _, _ = self._add_partial_measure(
                            qubits, cmems, cregs, err, kind, add_param)
                        break
                    elif exp_m:
                        data['Pauli_string_expectation'] = self._pauli_string_expectation(str(params[1]), err)
                        break
                    elif ensm:
                        spec = params[1]
                        if len(str(spec)) == 1:
                            add_param, basis = None, str(spec)
                        elif spec[0] == 'N':
                            add_param = self._unit_vector_normalisation(spec[1])
                            basis = 'N'
                        else:
                            raise BasicAerError('unrecognised ensemble basis %r' % (spec,))
                        prob, _, _ = self._add_ensemble_measure(basis, add_param, err)
                        data['ensemble_probability'] = prob
                        if self._counts_shots > 0:
                            cnt = self._dev.sample_counts(self._counts_shots, self._counts_seed)
                            data['counts'] = {k: int(c) for k, c in zip(prob, cnt) if c}
                        break
                else:
                    err_msg = '{0} encountered unrecognized operation "{1}"'
                    raise BasicAerError(err_msg.format(self.name(), name))
            self._add_decoherence_and_amp_decay(clock, f=mem['decoherence'], p=mem['thermalization'],
                                                g=mem['amplitude_decay'])
        trace_err = self._check_trace()
        if self.SHOW_FINAL_STATE and self._coefficients_to_host:
            if self._get_den_mat:
                data['coeffmatrix'], data['densitymatrix'] = self._get_densitymatrix()
            else:
                data['coeffmatrix'] = self._get_densitymatrix()
            if self._fidelity is not None:
                data['fidelity'] = self._fidelity
        if shadow_exp is not None:
            data.update(self._fp64_statement(shadow_exp, data))
            data['trace_err'] = trace_err
        self._dev.synchronize()
        end_runtime = time.time()
        self.last_run_stats = {'passes': self._dev.passes_run, 'levels': levels,
                               'kernel_launches': N.lib().dm_kernel_launch_count() - launches0,
                               'h2d_bytes': self._dev.h2d_bytes, 'd2h_bytes': self._dev.d2h_bytes,
                               'copy_out': dict(getattr(self._dev, 'copy_stats', {})),
                               'passes_by_kernel': dict(getattr(self._dev, 'passes_by_kernel', {})),
                               'composed_on': dict(getattr(self._dev, 'composed_on', {}))}
        if self._record_next:
            self.recorded_state = self._dev
            self._record_next = False
        self._dev = None
        return {'name': experiment.header.name,
                'number_of_clock_cycles': levels,
                'data': data,
                'status': 'DONE',
                'success': True,
                'processing_time_taken': -start_processing + end_processing,
                'running_time_taken': -start_runtime + end_runtime,
                'header': experiment.header.as_dict()}

    # ------------------------------------------------------- result checks
    TRACE_TOL = {'double': 1e-12, 'single': 1e-6}

    def _check_trace(self):
        """Trace preservation after the run: |2**n a_0 - 1| (a_0 read in FP64 on the device).

        The maps of every gate, channel and measurement keep a_0 = 2**-n
        (their I row is (1, 0, 0, 0)); a departure means the state was
        corrupted.  Same test as the reference's initial-state check
        (dm_simulator.py:363), applied to the final state."""
        err = self._dev.trace_error()
        if not err <= self.TRACE_TOL[self._precision]:
            raise BasicAerError('Trace of densitymatrix is not one after the run: |2^n a_0 - 1| = %.3g (> %g)'
                                % (err, self.TRACE_TOL[self._precision]))
        return err

    def _fp64_statement(self, experiment, data):
        """Error statement of an FP32 result: the same experiment run in FP64 on the device.

        Returns max_abs_coeff_err = max |2**n (a32 - a64)| over the final
        states (compared on the device) and prob_l1_err = the largest L1
        distance between a probability output of this run and the FP64 run's."""
        shadow = copy.copy(self)
        shadow._precision = 'double'
        shadow._fp64_check = False
        shadow._coefficients_to_host = False
        shadow._counts_shots = 0
        shadow._record_next = True
        shadow._dev = None
        ref = shadow.run_experiment(experiment)
        st64 = shadow.recorded_state
        n = self._number_of_qubits
        max_abs = self._dev.max_abs_diff(st64) * 2.0 ** n
        del st64
        shadow.recorded_state = None
        l1 = 0.0
        for k, v in ref['data'].items():
            g = data.get(k)
            if isinstance(v, dict) and isinstance(g, dict) and list(g.keys()) == list(v.keys()):
                a = np.array([float(x) for x in g.values()])
                b = np.array([float(x) for x in v.values()])
                l1 = max(l1, float(np.abs(a - b).sum()))
        return {'max_abs_coeff_err': max_abs, 'prob_l1_err': l1}

    # ---------------------------------------------------------------- outputs
    def _compute_densitymatrix(self, dmpauli=None):
        """dm_simulator.py:1198-1255, on the device."""
        return self._dev.density_matrix()

    def _get_densitymatrix(self):
        """dm_simulator.py:1257-1269: the matrix from the unchopped state, then the chopped vector."""
        if self._get_den_mat:
            densitymatrix = self._compute_densitymatrix()
            return self._dev.coefficients(self._chop_threshold), densitymatrix
        return self._dev.coefficients(self._chop_threshold)

    def _store_density_matrix(self):
        """dm_simulator.py:1271-1275."""
        np.save("stored_coefficients", self._dev.raw_coefficients())

    def _state_overlap(self, density_matrix_1, density_matrix_2=None):
        """dm_simulator.py:1277-1282: 2**n <a1, a2>, a2 being the device state when None."""
        if density_matrix_2 is None:
            return self._dev.overlap(density_matrix_1)
        return np.dot(density_matrix_1, density_matrix_2) * 2 ** self._number_of_qubits

    def _describe_partition(self, partition):
        """dm_simulator.py:1284-1313."""
        print("\nPARTITIONED CIRCUIT")
        for current in range(len(partition)):
            print("\nPartition ", current)
            for inst in partition[current]:
                name, qubit = inst.name, inst.qubits
                if name == 'u3':
                    print("U3", "   qubit", qubit, "    ", [round(float(x), 6) for x in inst.params])
                if name == 'u1':
                    print("U1", "   qubit", qubit, "    ", [round(float(x), 6) for x in inst.params])
                elif name == 'cx':
                    print("C-NOT", "   qubit", qubit)
                if name == 'measure':
                    if getattr(inst, 'params', None) is None:
                        setattr(inst, 'params', ['Z'])
                    param = inst.params
                    if param[0] == 'Bell' or str(param[0]) == 'Bell':
                        print('Bell Measure', "   qubit", [int(x) for x in str(param[1])])
                    else:
                        print(name, "   qubit", qubit, "    ", param)


def _u_decomposition(name, params):
    """basicaertools.py:69-90 (single_gate_dm_matrix)."""
    p = [float(x) for x in params]
    if name in ('U', 'u3'):
        return [['rz', p[2]], ['ry', p[0]], ['rz', p[1]]]
    if name == 'u1':
        return [['rz', p[0]]]
    raise QiskitError('Gate is not among the valid types: %s' % name)


def _bit_keys(m):
    import itertools
    return ["".join(s) for s in itertools.product("01", repeat=m)]
