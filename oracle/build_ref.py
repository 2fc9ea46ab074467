"""Build recipe for the reference pseudo-spectral kernel (test infrastructure).

This script is part of the oracle: it is used only by the tests, by
``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline leg, never by
the product path.

It compiles the reference's own hot path, ``pyqg/kernel.pyx`` (the Cython
``PseudoSpectralKernel``), from the file where it lies in the reference tree,
with the reference's numpy.fft fallback selected (``PYQG_USE_PYFFTW = 0``,
``pyqg/kernel.pyx:13-19,245-267``; pyFFTW/FFTW are not available here).  All
outputs go to ``oracle/_ref/`` which is git-ignored.

The reference tree is located by the environment variable
``PYQG_REFERENCE_ROOT`` (the directory holding ``pyqg/kernel.pyx``); without
it the stages that need the tree are skipped.

Three stages, so that the result can also be built on a machine without the
reference tree or Cython:

``cythonize``  needs the reference tree and Cython.  Writes
               ``oracle/_ref/pyqg_ref_kernel.c`` (generated C).
``stage``      needs the reference tree.  Copies the reference package's
               Python modules (``pyqg/*.py``, not its kernel) and its tests
               (``pyqg/tests``) to ``oracle/_ref/pyqg_src/pyqg/``, so that
               tests can run the unchanged ``pyqg.Model`` classes and the
               reference's own test suite over another kernel module on a
               machine without the tree.
``compile``    needs gcc, the Python headers and numpy.  Compiles that C file
               with ``-O3 -fopenmp`` (``setup.py:77-124`` of the reference uses
               ``-fopenmp`` the same way) into ``oracle/_ref/pyqg_ref_kernel*.so``.

Usage: ``python oracle/build_ref.py [cythonize] [stage] [compile]`` (all by
default).
"""
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("PYQG_REFERENCE_ROOT", "")
REF_KERNEL = os.path.join(REF_ROOT, "pyqg", "kernel.pyx") if REF_ROOT else ""
MODNAME = "pyqg_ref_kernel"
C_FILE = os.path.join(OUT, MODNAME + ".c")
STAGED = os.path.join(OUT, "pyqg_src")   # staged reference Python package


def tree_available():
    return bool(REF_KERNEL) and os.path.exists(REF_KERNEL)


def require_tree():
    if not REF_ROOT:
        raise FileNotFoundError("PYQG_REFERENCE_ROOT is not set: it must name the "
                                "directory that holds the reference's pyqg/kernel.pyx")
    if not os.path.exists(REF_KERNEL):
        raise FileNotFoundError("PYQG_REFERENCE_ROOT=%s holds no pyqg/kernel.pyx" % REF_ROOT)


def so_path():
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return os.path.join(OUT, MODNAME + suffix)


def cythonize():
    """Generate C from the reference kernel.pyx (numpy.fft fallback)."""
    require_tree()
    os.makedirs(OUT, exist_ok=True)
    inc = os.path.join(OUT, "include")
    os.makedirs(inc, exist_ok=True)
    # setup.py:67-75 of the reference generates this file at build time.
    with open(os.path.join(inc, ".compile_time_use_pyfftw.pxi"), "w") as f:
        f.write("DEF PYQG_USE_PYFFTW = 0\n")
    cmd = [sys.executable, "-m", "cython", "-3", "--module-name", MODNAME,
           "-I", inc, "-o", C_FILE, REF_KERNEL]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.PIPE)
    return C_FILE


def stage_python():
    """Copy the reference package's Python modules into oracle/_ref."""
    require_tree()
    src = os.path.join(REF_ROOT, "pyqg")
    dst = os.path.join(STAGED, "pyqg")
    if os.path.exists(dst):
        shutil.rmtree(dst)
    os.makedirs(dst)
    for name in sorted(os.listdir(src)):
        if name.endswith(".py"):
            shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
    # the reference's own tests and their fixtures (tests/reference_suite.py
    # runs them over a chosen kernel module)
    shutil.copytree(os.path.join(src, "tests"), os.path.join(dst, "tests"),
                    ignore=shutil.ignore_patterns("__pycache__", "*.pyc"))
    return dst


def staged_available():
    return os.path.exists(os.path.join(STAGED, "pyqg", "model.py"))


def compile_c():
    """Compile the generated C into an importable extension module."""
    import numpy as np
    if not os.path.exists(C_FILE):
        raise FileNotFoundError(C_FILE)
    pyinc = sysconfig.get_paths()["include"]
    if not os.path.exists(os.path.join(pyinc, "Python.h")):
        raise RuntimeError("Python.h not found in " + pyinc)
    out = so_path()
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared",
           "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
           "-I", pyinc, "-I", np.get_include(), C_FILE, "-o", out]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.PIPE)
    return out


def available():
    return os.path.exists(so_path())


def load():
    """Import the compiled reference kernel module (or raise ImportError)."""
    import importlib.util
    path = so_path()
    if not os.path.exists(path):
        raise ImportError("reference kernel not built: " + path)
    spec = importlib.util.spec_from_file_location(MODNAME, path)
    mod = importlib.util.module_from_spec(spec)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        spec.loader.exec_module(mod)
    return mod


def build(quiet=True):
    """Cythonize when the reference tree is present, then compile.

    Returns the path of the built module or None when it cannot be built.
    """
    try:
        if tree_available():
            cythonize()
            stage_python()
        if os.path.exists(C_FILE):
            return compile_c()
    except (subprocess.CalledProcessError, RuntimeError, OSError) as e:
        if not quiet:
            raise
        msg = getattr(e, "stderr", b"") or b""
        print("oracle/_ref build skipped:", e, msg.decode()[-400:],
              file=sys.stderr)
    return None


if __name__ == "__main__":
    stages = sys.argv[1:] or ["cythonize", "stage", "compile"]
    if "cythonize" in stages:
        print(cythonize())
    if "stage" in stages:
        print(stage_python())
    if "compile" in stages:
        print(compile_c())
