"""Load the reference's dm_simulator hot path (unmodified) with stubbed imports.

Used only by ``make_golden.py`` in a container that has the reference tree
checked out; nothing on the GPU machine, in ``bench.py`` or in the test suite
imports this module.

The reference package ``qiskit`` cannot be imported as a whole without
marshmallow / jsonschema / ply / matplotlib.  The two files on the hot path,
``qiskit/providers/basicaer/dm_simulator.py`` and
``qiskit/providers/basicaer/basicaertools.py``, only need a handful of names
from the rest of the package; this loader registers small stand-ins for those
names in ``sys.modules`` and then executes the two real files from the
reference tree by path.  ``sys.dont_write_bytecode`` is set so that nothing is
written into the (read-only) reference tree.
"""
import importlib.util
import os
import sys
import types

REF_ROOT = os.environ.get("DM_REFERENCE_ROOT", "/root/reference")
BASICAER = os.path.join(REF_ROOT, "qiskit", "providers", "basicaer")


class _Cfg(types.SimpleNamespace):
    @classmethod
    def from_dict(cls, d):
        return cls(**d)

    def to_dict(self):
        return dict(self.__dict__)


class _BaseBackend:
    def __init__(self, configuration, provider=None):
        self._configuration = configuration
        self._provider = provider

    def configuration(self):
        return self._configuration

    def name(self):
        return self._configuration.backend_name


class _QiskitError(Exception):
    pass


def _module(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    sys.modules[name] = m
    return m


def load():
    """Return the reference ``dm_simulator`` module (class ``DmSimulatorPy``)."""
    if "qiskit.providers.basicaer.dm_simulator" in sys.modules:
        return sys.modules["qiskit.providers.basicaer.dm_simulator"]
    sys.dont_write_bytecode = True
    pkg = _module("qiskit")
    pkg.__path__ = []
    _module("qiskit.exceptions", QiskitError=_QiskitError)
    _module("qiskit.util", local_hardware_info=lambda: {"memory": 64, "cpus": os.cpu_count()})
    prov = _module("qiskit.providers", BaseBackend=_BaseBackend)
    prov.__path__ = []
    _module("qiskit.providers.models", QasmBackendConfiguration=_Cfg)
    _module("qiskit.result", Result=dict)
    ba = _module("qiskit.providers.basicaer")
    ba.__path__ = [BASICAER]
    _module("qiskit.providers.basicaer.basicaerjob", BasicAerJob=object)

    class _BasicAerError(_QiskitError):
        pass

    _module("qiskit.providers.basicaer.exceptions", BasicAerError=_BasicAerError)
    plt = _module("matplotlib.pyplot")
    mpl = _module("matplotlib", pyplot=plt, cm=types.SimpleNamespace())
    mpl.__path__ = []
    tk = _module("mpl_toolkits")
    tk.__path__ = []
    _module("mpl_toolkits.mplot3d", Axes3D=object)

    for mod in ("basicaertools", "dm_simulator"):
        full = "qiskit.providers.basicaer." + mod
        spec = importlib.util.spec_from_file_location(full, os.path.join(BASICAER, mod + ".py"))
        m = importlib.util.module_from_spec(spec)
        sys.modules[full] = m
        spec.loader.exec_module(m)
    return sys.modules["qiskit.providers.basicaer.dm_simulator"]
