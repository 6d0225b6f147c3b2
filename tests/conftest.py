import importlib.util
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def _load_package():
    if 'qiskit_aakash_gb300' in sys.modules:
        return sys.modules['qiskit_aakash_gb300']
    d = os.path.join(REPO, 'qiskit-aakash_gb300')
    spec = importlib.util.spec_from_file_location(
        'qiskit_aakash_gb300', os.path.join(d, '__init__.py'), submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules['qiskit_aakash_gb300'] = m
    spec.loader.exec_module(m)
    return m


_load_package()


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a GB300 (runs the CUDA kernels)')
