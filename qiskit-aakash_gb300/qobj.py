"""Duck-typed qobj objects for the dm_simulator boundary.

The reference backend reads a ``QasmQobj`` built by qiskit's assembler
(qiskit/assembler/assemble_circuits.py:21-120).  Only attribute access is
used on it (dm_simulator.py:875-1196): ``qobj.config``, ``qobj.experiments``,
``qobj.qobj_id``, ``qobj.header.as_dict()``, and per experiment
``config.n_qubits``, ``config.memory_slots``, ``header.name`` and
``instructions[i].{name, qubits, params, memory, register, conditional}``.
These classes carry exactly those attributes, so that qobjs produced by the
reference's own assembler and qobjs produced here are interchangeable.

Instructions compare by identity, like the reference's marshmallow models
(qiskit/validation/base.py defines no ``__eq__``); the levelling pass relies
on that when it checks that a CX is on top of both of its qubit stacks.
"""
import copy
import uuid


class _Namespace:
    def __init__(self, **kw):
        self.__dict__.update(kw)

    def as_dict(self):
        out = {}
        for k, v in self.__dict__.items():
            out[k] = v.as_dict() if isinstance(v, _Namespace) else copy.deepcopy(v)
        return out

    to_dict = as_dict

    def __repr__(self):
        return '%s(%s)' % (type(self).__name__,
                           ', '.join('%s=%r' % kv for kv in self.__dict__.items()))


class QobjInstruction(_Namespace):
    """One qobj instruction (``QasmQobjInstruction`` fields)."""

    def __init__(self, name, qubits=None, params=None, memory=None, **kw):
        super().__init__(name=name, **kw)
        if qubits is not None:
            self.qubits = list(qubits)
        if params is not None:
            self.params = list(params)
        if memory is not None:
            self.memory = list(memory)


class QobjHeader(_Namespace):
    pass


class QobjConfig(_Namespace):
    pass


class QobjExperiment(_Namespace):
    def __init__(self, instructions, n_qubits, memory_slots=0, name='circuit0', header=None):
        super().__init__(
            instructions=list(instructions),
            config=QobjConfig(n_qubits=n_qubits, memory_slots=memory_slots),
            header=header if header is not None else QobjHeader(
                name=name, n_qubits=n_qubits, memory_slots=memory_slots))


class Qobj(_Namespace):
    def __init__(self, experiments, qobj_id=None, config=None, header=None):
        exps = list(experiments)
        nq = max([e.config.n_qubits for e in exps] or [0])
        ms = max([e.config.memory_slots for e in exps] or [0])
        super().__init__(
            experiments=exps,
            qobj_id=qobj_id or str(uuid.uuid4()),
            config=config if config is not None else QobjConfig(
                shots=1, memory_slots=ms, n_qubits=nq),
            header=header if header is not None else QobjHeader())
