"""Import the reference ``pyqg`` package in place (test infrastructure only).

Used by ``tests/golden/make_golden.py`` and by optional tests that compare
against the live reference in a container that has the reference tree.  The
reference's Python modules are imported from the reference tree itself; its
Cython kernel ``pyqg.kernel`` is provided by the module that
``oracle/build_ref.py`` compiled into ``oracle/_ref/``.  Bytecode writing is
disabled so nothing is written into the (read-only) reference tree.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("PYQG_REFERENCE_ROOT", "/root/reference")


def reference_available():
    return os.path.exists(os.path.join(REF_ROOT, "pyqg", "kernel.pyx"))


def import_reference_pyqg():
    """Return the reference ``pyqg`` module (building its kernel if needed)."""
    if "pyqg" in sys.modules and hasattr(sys.modules["pyqg"], "QGModel"):
        return sys.modules["pyqg"]
    if not reference_available():
        raise ImportError("reference tree not present")
    sys.path.insert(0, HERE)
    import build_ref
    if not build_ref.available():
        build_ref.build(quiet=False)
    sys.dont_write_bytecode = True
    kmod = build_ref.load()
    sys.modules["pyqg.kernel"] = kmod
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import pyqg  # noqa: E402  (the reference package)
    return pyqg
