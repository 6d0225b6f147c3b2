"""Exceptions with the reference's names and meanings.

``QiskitError`` (qiskit/exceptions.py) is raised for invalid gates and CX
labels (basicaertools.py:46, :88, :116, :338-339); ``BasicAerError``
(qiskit/providers/basicaer/exceptions.py) for invalid options, initial
states, unknown operations and qubit counts (dm_simulator.py:209-218, :315,
:880-882, :1167-1170).  When the reference package is importable, these are
the reference's own classes, so ``except BasicAerError`` works unchanged.
"""
try:  # pragma: no cover - exercised only where qiskit-aakash is installed
    from qiskit.exceptions import QiskitError  # noqa: F401
    from qiskit.providers.basicaer.exceptions import BasicAerError  # noqa: F401
except Exception:  # noqa: BLE001
    class QiskitError(Exception):
        """Base class for errors raised by this package."""

        def __init__(self, *message):
            super().__init__(' '.join(str(m) for m in message))
            self.message = ' '.join(str(m) for m in message)

    class BasicAerError(QiskitError):
        """Errors raised by the dm_simulator backend."""


class InitialStateError(BasicAerError, AttributeError):
    """Invalid initial density matrix.

    The reference's checks at dm_simulator.py:361 and :364 fail with an
    AttributeError while formatting their messages; this error is both a
    BasicAerError and an AttributeError, so handlers written for either see it.
    """
