"""CPU tests of the host side: the C ABI library loads and exports every
symbol declared in include/*.h (no compute calls), and the model constants
(grid, filter, inversion matrices, background) equal the reference's."""
import glob
import json
import os
import re

import numpy as np
import pytest

from conftest import REPO, golden


def header_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"\b(pqg_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    from pyqg_gb300 import _lib, build
    if not os.path.exists(build.lib_path()):
        build.build()
    return _lib.load()


def test_library_exports_every_header_symbol(lib):
    names = header_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_binding_signatures_cover_header():
    from pyqg_gb300 import _lib
    assert header_symbols() == set(_lib.SIGNATURES)


def test_library_reports_version_and_errors(lib):
    assert lib.pqg_version() >= 100
    assert lib.pqg_plan_create(None, 2, 64, 64) == 1   # PQG_ERR_INVALID, no GPU touched
    assert b"NULL" in lib.pqg_last_error()


def test_product_refuses_to_run_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    import pyqg_gb300 as P
    with pytest.raises(RuntimeError, match="CUDA"):
        P.QGModel()


def test_parameterization_entry_points_refuse_bad_arguments():
    """The pointwise parameterization stages check their arguments on the
    host and report PQG_ERR_INVALID with the entry point's name before any
    CUDA call (so this runs without a GPU)."""
    from pyqg_gb300 import _lib
    L = _lib.lib()
    x = 8   # a non-null placeholder address: the checks reject the call first
    cases = {
        "pqg_smag_strain": (0, 8, 5, x, x, x, x, x, None),
        "pqg_smag_stress": (2, 8, 8, x, 1.0, None, None, None),
        "pqg_smag_divergence": (2, 8, 5, x, x, None, x, None),
        "pqg_zb_gradients": (2, 0, 5, x, x, x, x, x, None),
        "pqg_zb_products": (2, 8, 8, None, x, None),
        "pqg_zb_combine": (2, 8, 5, x, x, x, 1.0, None, None),
        "pqg_lap_power": (2, 8, 5, x, x, 3, 1.0, x, x, None),
        "pqg_layer_mix": (9, 2, 64, x, x, x, None),
        "pqg_mul_scaled": (0, x, 1.0, x, x, None),
        "pqg_backscatter": (2, 8, 8, x, x, x, None, 1.0, 1e-32, x, x, None),
        "pqg_ring_normalize": (1, 8, 8, x, None, 1.0, x, x, None),
    }
    for name, args in cases.items():
        rc = getattr(L, name)(*args)
        assert rc == _lib.PQG_ERR_INVALID, name
        assert name in L.pqg_last_error().decode(), name


def _qg_consts(n, L=1e6, rd=15000.0, delta=0.25, beta=1.5e-11, U1=0.025,
               U2=0.0, filterfac=23.6):
    from pyqg_gb300.model import grid_constants, spectral_filter
    from pyqg_gb300.qg_model import qg_inversion_matrix
    g = grid_constants(n, n, L, L)
    F1 = rd ** -2 / (1. + delta)
    F2 = delta * F1
    return dict(a=qg_inversion_matrix(g["wv2"], F1, F2), kk=g["kk"], ll=g["ll"],
                filtr=spectral_filter(g["k"], g["l"], g["dx"], g["dy"], filterfac),
                Qy=np.array([beta + F1 * (U1 - U2), beta - F2 * (U1 - U2)]))


def test_qg_constants_equal_reference():
    g = golden("qg_two_layer_nx64.npz")
    c = _qg_consts(64)
    for k in ("a", "kk", "ll", "Qy"):
        np.testing.assert_array_equal(c[k], g[k], err_msg=k)
    # libm exp may differ by an ulp between hosts
    np.testing.assert_allclose(c["filtr"], g["filtr"], rtol=1e-14, atol=0)


def test_layered_constants_equal_reference():
    from pyqg_gb300.model import grid_constants, spectral_filter
    from pyqg_gb300.layered_model import stretching_matrix, layered_inversion_matrix
    g = golden("layered_nz3_nx32.npz")
    grid = grid_constants(32, 32, 1e6, 1e6)
    rho = np.arange(3) * 0.3 + 1025
    gpi = 9.81 * (rho[1:] - rho[:-1]) / rho[:-1]
    f = 0.0001236812857687059
    S = stretching_matrix(3, f ** 2, np.array([500., 1000., 2500.]), gpi)
    a = layered_inversion_matrix(S, grid["wv2"])
    np.testing.assert_allclose(a, g["a"], rtol=1e-15, atol=0)
    Qy = 1.5e-11 - S @ np.array([0.05, 0.02, 0.0])
    np.testing.assert_allclose(Qy, g["Qy"], rtol=1e-15)
    np.testing.assert_allclose(
        spectral_filter(grid["k"], grid["l"], grid["dx"], grid["dy"], 23.6), g["filtr"],
        rtol=1e-14, atol=0)


def test_layered_fixture_params_constants():
    """The reference's own LayeredModel test fixture parameters (nx=64)."""
    from pyqg_gb300.model import grid_constants
    from pyqg_gb300.layered_model import stretching_matrix, layered_inversion_matrix
    g = golden("layered_fixture_nx64.npz")
    p = json.loads(str(g["params_json"]))
    grid = grid_constants(64, 64, p["L"], p["L"])
    rho = np.array(p["rho"])
    gpi = p["g"] * (rho[1:] - rho[:-1]) / rho[:-1]
    S = stretching_matrix(3, p["f"] ** 2, np.array(p["H"], dtype=float), gpi)
    np.testing.assert_allclose(layered_inversion_matrix(S, grid["wv2"]), g["a"],
                               rtol=1e-14, atol=0)


def test_stretching_matrix_properties():
    """S has zero row sums and H S is symmetric (pyqg/tests/test_layered.py)."""
    from pyqg_gb300.layered_model import stretching_matrix
    Hi = np.array([.1, .1, .3])
    rho = np.array([.1, .3, .5])
    gpi = 9.81 * (rho[1:] - rho[:-1]) / rho[:-1]
    S = stretching_matrix(3, 1.0, Hi, gpi)
    assert np.all(S.sum(axis=1) == 0.)
    HS = np.diag(Hi) @ S
    np.testing.assert_allclose(HS, HS.T, atol=1e-16)


def test_single_layer_inversions():
    from pyqg_gb300.model import grid_constants
    for case in ("bt_nx32.npz", "sqg_nx32.npz"):
        g = golden(case)
        grid = grid_constants(32, 32, 2 * np.pi, 2 * np.pi)
        if case.startswith("bt"):
            a = -grid["wv2i"][np.newaxis, np.newaxis]
        else:
            a = np.sqrt(grid["wv2i"])[np.newaxis, np.newaxis]
        np.testing.assert_array_equal(a, g["a"])


def test_parameterization_algebra():
    import pyqg_gb300 as P
    smag, zb = P.Smagorinsky(), P.ZannaBolton2020()
    comb = 0.5 * smag + 0.75 * zb
    assert comb.parameterization_type == "uv_parameterization"
    with pytest.raises(AssertionError):
        P.BackscatterBiharmonic() + smag


class _FakeModel:
    """Host-side stand-in with the attributes the batching logic reads."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def test_fused_run_length_stops_at_observation_points():
    from pyqg_gb300.model import Model
    m = _FakeModel(t=0.0, tc=0, dt=10.0, tmax=1e9, tavestart=1e30, taveints=1.0,
                   log_level=1, twrite=25, q_parameterization=None,
                   uv_parameterization=None)
    m._fusable = lambda: True
    m._diagnostics_due = lambda t, tc: Model._diagnostics_due(m, t, tc)
    m._status_due = lambda tc: Model._status_due(m, tc)
    # status every 25 steps: the first batch ends after step 25
    assert Model._fusable_run_length(m) == 25
    m.tc, m.t = 25, 250.0
    assert Model._fusable_run_length(m) == 25
    # tmax cuts the batch
    m.tmax = 300.0
    assert Model._fusable_run_length(m) == 5
    # diagnostics due now: no fused step
    m.tmax, m.tavestart = 1e9, 0.0
    assert Model._fusable_run_length(m) == 0
    # a snapshot predicate ends the batch after the matching step
    m.tavestart, m.log_level = 1e30, 0
    assert Model._fusable_run_length(m, lambda t, tc: tc % 7 == 0) == 3


def test_model_refuses_non_square_grid():
    """The reference's model grid builds ll from nx (pyqg/model.py:459-460):
    the model classes refuse ny != nx before touching the device."""
    import pytest
    import pyqg_gb300 as P
    with pytest.raises(ValueError, match="ny != nx"):
        P.QGModel(nx=64, ny=32, log_level=0)


def test_header_compiles_as_c_and_links(tmp_path):
    """include/pyqg_gb300.h is plain C99 (the reference-side FFI binds it
    from C): a C program compiles against it, links the library and calls
    entry points that need no GPU."""
    import os
    import shutil
    import subprocess
    import pytest
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.join(root, "pyqg_gb300", "lib")
    if not os.path.exists(os.path.join(libdir, "libpyqg_gb300.so")):
        pytest.skip("library not built")
    src = tmp_path / "use_header.c"
    src.write_text('#include "pyqg_gb300.h"\n#include <stdio.h>\n'
                   'int main(void) {\n'
                   '  int v = pqg_version();\n'
                   '  const char *e = pqg_last_error();\n'
                   '  printf("%d %d\\n", v > 0, e != 0);\n'
                   '  return 0;\n}\n')
    exe = tmp_path / "use_header"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                    os.path.join(root, "include"), str(src), "-L", libdir, "-lpyqg_gb300",
                    "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert out == ["1", "1"]


def test_reference_arm_prints_its_json_line():
    """`bench.py --impl reference` runs on the host alone: one JSON line with
    the metric, impl, cpu_baseline (kind, cores, sample), e2e and no GPU
    launches."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "1", "--chunk", "5"],
                         cwd=root, check=True, capture_output=True, text=True, timeout=600).stdout
    line = json.loads(out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "sim-yr/hr" and line["value"] > 0
    assert line["gpu_launches"] == 0
    assert set(line["cpu_baseline"]) >= {"value", "unit", "cores", "kind", "sample"}
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]


def test_bench_measurement_definitions():
    """The bench's units: compulsory FP64 bytes per model step B64 = 80 S +
    16 P (S spectral, P grid points; 468,992 B at nx=64 and 7,380,992 B at
    nx=256 for two layers, 703,488 B and 11,071,488 B for three), a year of
    360 days (pyqg/tests/test_reference_solns.py:12), and the stored ncu
    traffic labelled with the capture that made it."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.algorithmic_bytes(2, 64, 64) == 468992
    assert bench.algorithmic_bytes(2, 256, 256) == 7380992
    assert bench.algorithmic_bytes(3, 64, 64) == 703488
    assert bench.algorithmic_bytes(3, 256, 256) == 11071488
    # one year of dt = 3600 s steps in one hour of wall time is 1 sim-yr/hr
    assert abs(bench.sim_yr_per_hr(360 * 24, 3600.0, 3600.0) - 1.0) < 1e-12
    for name in ("k_col_fused_fx", "k_row_adv_fx", "ensemble_1024_mixed_step"):
        nbytes, src = bench.stored_traffic(name)
        assert nbytes > 0 and src.startswith("stored ncu capture: ncu ") and "--clock-control none" in src


def test_closure_experiment_truncation_matches_the_coarse_oracle():
    """The experiment's host truncation of physical PV (used for the coarse
    runs' initial states) is the coarse-graining oracle's sharp cutoff:
    |k|, |l| < nc / 2 kept, amplitudes rescaled to the coarse grid."""
    from coarse_oracle import truncate
    from pyqg_oracle import irfft2, rfft2
    from pyqg_gb300.closure_experiment import _truncate_physical
    rng = np.random.default_rng(17)
    for nf, nc in ((64, 32), (256, 64), (96, 32)):
        q = rng.standard_normal((2, nf, nf))
        got = _truncate_physical(q, nc)
        want = irfft2(truncate(rfft2(q), nc, nc))
        assert got.shape == (2, nc, nc)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * np.abs(want).max())
        # idempotent: a truncated field is kept as it is
        np.testing.assert_allclose(_truncate_physical(got, nc), got, rtol=0, atol=1e-13 * np.abs(got).max())
