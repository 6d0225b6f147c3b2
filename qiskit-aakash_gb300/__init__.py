"""GB300-native engine for qiskit-aakash's ``dm_simulator`` hot path.

The density matrix is a real vector of 4**n Pauli-basis coefficients kept in
GB300 HBM; gates, noise channels and measurements are applied by hand-written
sm_103a CUDA kernels reached through the C-ABI library ``libdmgb300.so``
(include/dm_gb300.h).  The public surface mirrors the reference backend
(qiskit/providers/basicaer/dm_simulator.py:61-1313): ``DmSimulatorGPU``
(``run``, ``_run_job``, ``run_experiment``), the ``BasicAer`` provider lookup
by the name ``'dm_simulator'`` and ``execute``.
"""
from .circuit import QuantumCircuit, noise_options, random_layer_circuit  # noqa: F401
from .exceptions import BasicAerError, QiskitError  # noqa: F401
from .qobj import Qobj, QobjExperiment, QobjInstruction  # noqa: F401


def __getattr__(name):
    # The backend, provider and execute import the engine lazily so that the
    # circuit/qobj helpers stay importable without a GPU or a built library.
    if name in ('DmSimulatorGPU', 'DmGpuJob'):
        from . import dm_simulator
        return getattr(dm_simulator, name)
    if name in ('BasicAer', 'execute', 'assemble', 'DmGpuProvider'):
        from . import provider
        return getattr(provider, name)
    if name == 'build':
        from ._native import build
        return build
    raise AttributeError(name)
