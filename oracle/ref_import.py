"""Import the reference ``pyqg`` package (test infrastructure only).

Two uses, both by tests and by ``tests/golden/make_golden.py``, never by the
product path:

``import_reference_pyqg()``
    The reference package in place, from the tree named by the environment
    variable ``PYQG_REFERENCE_ROOT``, with its Cython kernel ``pyqg.kernel``
    provided by the module that ``oracle/build_ref.py`` compiled into
    ``oracle/_ref/``.  Bytecode writing is disabled so nothing is written
    into the (read-only) reference tree.

``import_reference_on(kernel_module)``
    The reference's unchanged Python modules, staged by
    ``oracle/build_ref.py`` into ``oracle/_ref/pyqg_src/`` (so no reference
    tree is needed at run time), with ``kernel_module`` standing in for its
    compiled ``pyqg.kernel``.  This is how pyqg would load a replacement
    kernel: ``pyqg/model.py:8`` imports ``PseudoSpectralKernel`` and the
    ``tendency_*`` helpers from ``.kernel``.  The package is returned and
    the ``pyqg`` entries of ``sys.modules`` are put back as they were, so
    it does not clash with another ``pyqg`` loaded in the same process.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("PYQG_REFERENCE_ROOT", "")


def reference_available():
    return bool(REF_ROOT) and os.path.exists(os.path.join(REF_ROOT, "pyqg", "kernel.pyx"))


def staged_available():
    sys.path.insert(0, HERE)
    import build_ref
    return build_ref.staged_available()


def import_reference_pyqg():
    """Return the reference ``pyqg`` module (building its kernel if needed)."""
    if "pyqg" in sys.modules and hasattr(sys.modules["pyqg"], "QGModel"):
        return sys.modules["pyqg"]
    if not reference_available():
        raise ImportError("reference tree not present: set PYQG_REFERENCE_ROOT to the "
                          "directory that holds pyqg/kernel.pyx")
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


def _pyqg_entries():
    return {k: v for k, v in sys.modules.items() if k == "pyqg" or k.startswith("pyqg.")}


def import_reference_on(kernel_module):
    """The staged, unchanged reference package over ``kernel_module``."""
    sys.path.insert(0, HERE)
    import build_ref
    if not build_ref.staged_available():
        raise ImportError("reference package not staged: run oracle/build_ref.py "
                          "with PYQG_REFERENCE_ROOT set")
    saved = _pyqg_entries()
    for k in saved:
        del sys.modules[k]
    src = build_ref.STAGED
    sys.modules["pyqg.kernel"] = kernel_module
    sys.path.insert(0, src)
    old_bc = sys.dont_write_bytecode
    sys.dont_write_bytecode = True
    try:
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            import pyqg  # noqa: E402  (the staged reference package)
        pkg = pyqg
    finally:
        sys.dont_write_bytecode = old_bc
        sys.path.remove(src)
        for k in _pyqg_entries():
            del sys.modules[k]
        sys.modules.update(saved)
    return pkg
