"""Run the reference's own test suite, unchanged, over a chosen kernel
module (test infrastructure).

    python tests/reference_suite.py --kernel gpu|stock --out outcomes.json

The reference's Python modules and its ``pyqg/tests`` are the copies that
``oracle/build_ref.py`` staged into ``oracle/_ref/pyqg_src`` (no reference
tree is needed at run time).  ``--kernel gpu`` registers
``pyqg_gb300.kernel`` as ``pyqg.kernel``; ``--kernel stock`` the reference's
compiled Cython kernel.  The reference's tests import
``future.utils.iteritems`` (a Python-2 compatibility package that is not
installed); the runner provides that one function in memory.  The outcome
of every test (passed / failed / skipped) is written as JSON.
"""
import argparse
import json
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", choices=["gpu", "stock"], required=True)
    ap.add_argument("--out", required=True)
    ap.add_argument("pytest_args", nargs="*")
    a = ap.parse_args(argv)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    sys.path.insert(0, REPO)
    import build_ref
    staged = build_ref.STAGED
    tests = os.path.join(staged, "pyqg", "tests")
    if not os.path.isdir(tests):
        raise SystemExit("reference tests not staged: run oracle/build_ref.py with PYQG_REFERENCE_ROOT")
    fut = types.ModuleType("future")
    fut_utils = types.ModuleType("future.utils")
    fut_utils.iteritems = lambda d: iter(d.items())
    fut.utils = fut_utils
    sys.modules["future"] = fut
    sys.modules["future.utils"] = fut_utils
    if a.kernel == "gpu":
        import pyqg_gb300.kernel as kmod
    else:
        kmod = build_ref.load()
    sys.modules["pyqg.kernel"] = kmod
    sys.path.insert(0, staged)
    sys.dont_write_bytecode = True
    import pyqg  # the staged reference package over the chosen kernel
    assert pyqg.model.PseudoSpectralKernel is kmod.PseudoSpectralKernel

    outcomes = {}

    class Recorder:
        def pytest_runtest_logreport(self, report):
            if report.when == "call" or (report.when == "setup" and report.outcome != "passed"):
                outcomes[report.nodeid] = report.outcome

    import pytest
    os.chdir(tests)   # the reference's tests open their fixtures by relative path
    # test_xarray_output.py imports xarray at module level; xarray is not
    # installed, so that module cannot be collected
    rc = pytest.main([tests, "-q", "-p", "no:cacheprovider", "-W", "ignore",
                      "--ignore=" + os.path.join(tests, "test_xarray_output.py")] + a.pytest_args,
                     plugins=[Recorder()])
    with open(a.out, "w") as f:
        json.dump({"kernel": a.kernel, "outcomes": outcomes}, f, indent=1, sort_keys=True)
    return int(rc) if int(rc) in (0, 1) else int(rc)


if __name__ == "__main__":
    sys.exit(main())
