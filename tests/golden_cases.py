"""Read the golden fixtures written by tests/golden/make_golden.py."""
import json
import os

import numpy as np
import sympy

import qiskit_aakash_gb300 as dmg

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
_CACHE = {}


def _load():
    if not _CACHE:
        with open(os.path.join(GOLDEN, 'cases.json')) as f:
            _CACHE['cases'] = json.load(f)['cases']
        _CACHE['arrays'] = dict(np.load(os.path.join(GOLDEN, 'outputs.npz')))
    return _CACHE['cases'], _CACHE['arrays']


def cases(tag=None):
    cs, _ = _load()
    return [c for c in cs if tag is None or tag in c['tags']]


def case(name):
    for c in cases():
        if c['name'] == name:
            return c
    raise KeyError(name)


def array(key):
    return _load()[1][key]


def dec_param(p):
    if 's' in p:
        return sympy.Symbol(p['s'])
    if 'a' in p:
        return np.array(p['a'], dtype=float)
    if 'l' in p:
        return [dec_param(x) for x in p['l']]
    if 'str' in p:
        return p['str']
    return p['f']


def instructions(c):
    out = []
    for d in c['instructions']:
        kw = {k: v for k, v in d.items() if k not in ('name', 'params')}
        inst = dmg.QobjInstruction(d['name'], **kw)
        if 'params' in d:
            inst.params = [dec_param(p) for p in d['params']]
        out.append(inst)
    return out


def experiment(c):
    return dmg.QobjExperiment(instructions(c), c['n'], c['memory_slots'], name=c['name'])


def options(c):
    import copy
    return copy.deepcopy(c['options'])
