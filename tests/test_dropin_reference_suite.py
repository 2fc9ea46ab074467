"""The reference's own test suite, unchanged, over the GPU kernel.

``tests/reference_suite.py`` runs the reference's ``pyqg/tests`` (staged by
``oracle/build_ref.py``) with ``pyqg_gb300.kernel`` registered as
``pyqg.kernel``: pyqg's unchanged model classes, diagnostics and
parameterizations then step on the GPU.  The stock Cython kernel's outcomes
on the same files (``tests/golden/reference_suite_stock.json``, written by
``python tests/reference_suite.py --kernel stock --out ...`` in a container
with the reference tree) are the bar: every test the stock kernel passes
must pass, and the GPU kernel may fail only where the stock kernel fails
(five tests that call ``np.linalg.solve`` in a form numpy 2 rejects,
``pyqg/model.py:313``).  ``test_xarray_output.py`` is not collected:
xarray is not installed.
"""
import json
import os
import subprocess
import sys

import pytest

from conftest import GOLDEN, REPO

pytestmark = pytest.mark.gpu


def test_reference_suite_over_gpu_kernel(tmp_path):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import build_ref
    if not os.path.isdir(os.path.join(build_ref.STAGED, "pyqg", "tests")):
        pytest.skip("reference tests not staged (oracle/build_ref.py with PYQG_REFERENCE_ROOT)")
    out = tmp_path / "gpu.json"
    res = subprocess.run([sys.executable, os.path.join(REPO, "tests", "reference_suite.py"),
                          "--kernel", "gpu", "--out", str(out)],
                         capture_output=True, text=True, timeout=1800)
    assert out.exists(), res.stdout[-3000:] + res.stderr[-3000:]
    gpu = json.loads(out.read_text())["outcomes"]
    with open(os.path.join(GOLDEN, "reference_suite_stock.json")) as f:
        stock = json.load(f)["outcomes"]
    assert set(gpu) == set(stock), sorted(set(gpu) ^ set(stock))
    regressions = [t for t, o in stock.items() if o == "passed" and gpu[t] != "passed"]
    assert not regressions, (regressions, res.stdout[-4000:])
    extra_failures = [t for t, o in gpu.items() if o == "failed" and stock[t] != "failed"]
    assert not extra_failures, extra_failures
    assert sum(o == "passed" for o in gpu.values()) >= 54
