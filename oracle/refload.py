"""Load the reference's dm_simulator hot path (unmodified) with stubbed imports.

Test infrastructure: used by the golden-fixture scripts under ``tests/golden/``
and by ``bench.py``'s CPU legs to time the reference itself.  No product code
imports it.

The reference package ``qiskit`` (qiskit-terra 0.9.0 with the added
``dm_simulator`` backend) cannot be imported as a whole without marshmallow /
jsonschema / ply / matplotlib.  The two files on the hot path,
``qiskit/providers/basicaer/dm_simulator.py`` and
``qiskit/providers/basicaer/basicaertools.py``, need only a handful of names
from the rest of the package; this loader registers small stand-ins for those
names in ``sys.modules`` and then executes the two real files.

Two sources are accepted:

* the reference tree itself (``ref_root`` argument or the ``DM_REFERENCE_ROOT``
  environment variable), executing the ``.py`` files where they lie;
* the byte-compiled copies that ``oracle/build_ref.py`` writes into
  ``oracle/_ref/`` (``basicaertools.pyc``, ``dm_simulator.pyc``), for a
  machine that has no reference tree.  Byte code is the same on every
  platform for one Python minor version; the loader checks that version.

``sys.dont_write_bytecode`` is set so that nothing is written into the
(read-only) reference tree.
"""
import importlib.machinery
import importlib.util
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
PYC_DIR = os.path.join(HERE, '_ref')
MODULES = ('basicaertools', 'dm_simulator')
_PKG = 'qiskit.providers.basicaer'


class ReferenceUnavailable(RuntimeError):
    """Neither a reference tree nor its byte-compiled copies are present."""


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


def basicaer_dir(ref_root=None):
    """The reference's ``qiskit/providers/basicaer`` directory, or None."""
    root = ref_root or os.environ.get('DM_REFERENCE_ROOT')
    if not root:
        return None
    d = os.path.join(root, 'qiskit', 'providers', 'basicaer')
    return d if all(os.path.isfile(os.path.join(d, m + '.py')) for m in MODULES) else None


def pyc_path(mod):
    return os.path.join(PYC_DIR, mod + '.pyc')


def available(ref_root=None):
    """Where the reference can be loaded from: 'source', 'pyc' or None."""
    if basicaer_dir(ref_root):
        return 'source'
    if all(os.path.isfile(pyc_path(m)) for m in MODULES) and _pyc_version_ok():
        return 'pyc'
    return None


def _pyc_version_ok():
    magic = importlib.util.MAGIC_NUMBER
    try:
        with open(pyc_path(MODULES[0]), 'rb') as f:
            return f.read(len(magic)) == magic
    except OSError:
        return False


def _install_stubs(search_dir):
    pkg = _module('qiskit')
    pkg.__path__ = []
    _module('qiskit.exceptions', QiskitError=_QiskitError)
    _module('qiskit.util', local_hardware_info=lambda: {'memory': 64, 'cpus': os.cpu_count()})
    prov = _module('qiskit.providers', BaseBackend=_BaseBackend)
    prov.__path__ = []
    _module('qiskit.providers.models', QasmBackendConfiguration=_Cfg)
    _module('qiskit.result', Result=dict)
    ba = _module(_PKG)
    ba.__path__ = [search_dir]
    _module(_PKG + '.basicaerjob', BasicAerJob=object)

    class _BasicAerError(_QiskitError):
        pass

    _module(_PKG + '.exceptions', BasicAerError=_BasicAerError)
    plt = _module('matplotlib.pyplot')
    mpl = _module('matplotlib', pyplot=plt, cm=types.SimpleNamespace())
    mpl.__path__ = []
    tk = _module('mpl_toolkits')
    tk.__path__ = []
    _module('mpl_toolkits.mplot3d', Axes3D=object)


def load(ref_root=None):
    """Return the reference ``dm_simulator`` module (class ``DmSimulatorPy``).

    Raises ReferenceUnavailable when neither form of the reference is present.
    """
    full = _PKG + '.dm_simulator'
    if full in sys.modules:
        return sys.modules[full]
    sys.dont_write_bytecode = True
    src = basicaer_dir(ref_root)
    if src is None and available() != 'pyc':
        raise ReferenceUnavailable(
            'the reference dm_simulator is not available: set DM_REFERENCE_ROOT to the reference tree, '
            'or build oracle/_ref with oracle/build_ref.py where the tree exists')
    _install_stubs(src or PYC_DIR)
    for mod in MODULES:
        name = _PKG + '.' + mod
        if src is not None:
            spec = importlib.util.spec_from_file_location(name, os.path.join(src, mod + '.py'))
        else:
            loader = importlib.machinery.SourcelessFileLoader(name, pyc_path(mod))
            spec = importlib.util.spec_from_loader(name, loader)
        m = importlib.util.module_from_spec(spec)
        sys.modules[name] = m
        spec.loader.exec_module(m)
    return sys.modules[full]
