"""GB300-native engine for qiskit-aakash's ``dm_simulator`` hot path.

The density matrix is a real vector of 4**n Pauli-basis coefficients kept in
GB300 HBM; gates, noise channels and measurements are applied by hand-written
sm_103a CUDA kernels reached through the C-ABI library ``libdmgb300.so``.
The public surface mirrors the reference backend (dm_simulator.py:61-1313):
``DmSimulatorGPU`` (``run``, ``_run_job``, ``run_experiment``), the
``BasicAer`` provider lookup by the name ``'dm_simulator'`` and ``execute``.
"""
from .circuit import QuantumCircuit, random_layer_circuit, noise_options  # noqa: F401
from .qobj import Qobj, QobjExperiment, QobjInstruction  # noqa: F401
