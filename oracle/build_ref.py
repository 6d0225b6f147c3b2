"""Recipe: byte-compile the reference's two hot-path files into ``oracle/_ref/``.

The reference is Python (``qiskit/providers/basicaer/basicaertools.py`` and
``qiskit/providers/basicaer/dm_simulator.py``).  Compiling them to ``.pyc``
files lets ``oracle/refload.py`` run the unmodified reference on a machine
that has no reference tree (the CPU legs of ``bench.py`` time it there).
``oracle/_ref/`` is git-ignored: nothing of the reference enters the
repository's history.

Usage: ``python oracle/build_ref.py [REFERENCE_ROOT]``; the root defaults to
``DM_REFERENCE_ROOT`` or ``/root/reference``.  Does nothing when the tree is
absent (the prebuilt files, if any, are kept).
"""
import os
import py_compile
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import refload  # noqa: E402


def build(ref_root=None, verbose=False):
    root = ref_root or os.environ.get('DM_REFERENCE_ROOT') or '/root/reference'
    src = refload.basicaer_dir(root)
    if src is None:
        if verbose:
            print('oracle/_ref: no reference tree at %s; keeping %s' % (root, refload.available() or 'nothing'))
        return False
    os.makedirs(refload.PYC_DIR, exist_ok=True)
    for mod in refload.MODULES:
        py_compile.compile(os.path.join(src, mod + '.py'), cfile=refload.pyc_path(mod), doraise=True,
                           invalidation_mode=py_compile.PycInvalidationMode.UNCHECKED_HASH)
    if verbose:
        print('oracle/_ref: byte-compiled %s from %s' % (', '.join(refload.MODULES), src))
    return True


if __name__ == '__main__':
    build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True)
