"""Provider lookup and ``execute`` for the GB300 dm_simulator.

``BasicAer.get_backend('dm_simulator')`` resolves the backend by its
configured name, as the reference's provider does
(qiskit/providers/basicaer/basicaerprovider.py:51-66), including the
deprecated alias ``dm_simulator_py`` (:94).  ``execute`` takes circuits
built with this package's ``QuantumCircuit`` (already in the backend's
basis) or a ready qobj, and forwards its keyword arguments as
``backend_options`` exactly like qiskit/execute.py:204.
"""
from .circuit import QuantumCircuit
from .dm_simulator import DmSimulatorGPU
from .exceptions import QiskitError
from .qobj import Qobj

_ALIASES = {'dm_simulator_py': 'dm_simulator'}


class DmGpuProvider:
    """Holds one instance of each backend class, like BasicAerProvider."""

    SIMULATORS = [DmSimulatorGPU]

    def __init__(self):
        self._backends = {}
        for cls in self.SIMULATORS:
            b = cls(provider=self)
            self._backends[b.name()] = b

    def backends(self, name=None, **kwargs):
        if name:
            name = _ALIASES.get(name, name)
            return [b for b in self._backends.values() if b.name() == name]
        return list(self._backends.values())

    def get_backend(self, name=None, **kwargs):
        found = self.backends(name, **kwargs)
        if not found:
            raise QiskitError("The '{}' backend is not installed in your system.".format(name))
        return found[0]

    def __str__(self):
        return 'BasicAer'


BasicAer = DmGpuProvider()


def assemble(experiments, qobj_id=None):
    """Build a qobj from circuits (or return a qobj unchanged)."""
    if isinstance(experiments, Qobj):
        return experiments
    if isinstance(experiments, QuantumCircuit):
        experiments = [experiments]
    return Qobj([c.to_experiment() if isinstance(c, QuantumCircuit) else c for c in experiments],
                qobj_id=qobj_id)


def execute(experiments, backend, qobj_id=None, **run_config):
    """Run circuits on ``backend``; keyword arguments become backend options."""
    qobj = assemble(experiments, qobj_id=qobj_id)
    return backend.run(qobj, backend_options={**run_config})
