"""ctypes binding of ``libpyqg_gb300.so`` (the C ABI in include/pyqg_gb300.h).

The library is built in-tree by ``pyqg_gb300.build``; importing this module
never falls back to any other implementation: if the library is missing or
fails to load, :func:`lib` raises.
"""
import ctypes
import os
import threading

from .build import lib_path

PQG_OK = 0
PQG_ERR_INVALID = 1
PQG_ERR_UNSUPPORTED = 2
PQG_ERR_CUDA = 3
PQG_ERR_NOMEM = 4
PQG_ERR_STATE = 5
PQG_ERR_TIMEOUT = 6
PQG_NOALLOC_MAX_COMPLEX = 1 << 19   # scratch limit of pqg_rfft2_noalloc

_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int


class Aux(ctypes.Structure):
    _fields_ = [(n, _P) for n in ("ph", "uh", "vh", "u", "v", "uq", "vq",
                                  "uqh", "vqh")]


class State(ctypes.Structure):
    _fields_ = [("q", _P), ("qh", _P), ("dqhdt", _P), ("dqhdt_p", _P),
                ("dqhdt_pp", _P), ("ablevel", _I), ("tc", ctypes.c_longlong),
                ("t", _D), ("dt", _D)]


_PD = ctypes.POINTER(ctypes.c_double)


class DiagFields(ctypes.Structure):
    """pqg_diag_fields (include/pyqg_gb300.h)."""
    _fields_ = ([(n, _PD) for n in ("qh", "ph", "dqhdt", "dqhdt_p", "dqhdt_pp", "u", "v", "Jq",
                                    "Jpxi", "Jptpc", "JSp", "Sph", "phn", "dqh", "duh", "dvh")] +
                [(n, _D) for n in ("H", "dt", "c1", "c2", "c3", "rd", "del1", "del2", "U")] +
                [(n, _PD) for n in ("Hi", "Qx", "Qy", "Ubg", "Vbg", "f2gpi", "kdi2", "S")])


# name -> (restype, argtypes)
SIGNATURES = {
    "pqg_version": (_I, []),
    "pqg_last_error": (ctypes.c_char_p, []),
    "pqg_plan_create": (_I, [ctypes.POINTER(_P), _I, _I, _I]),
    "pqg_plan_destroy": (_I, [_P]),
    "pqg_set_wavenumbers": (_I, [_P, _P, _P]),
    "pqg_set_k2l2": (_I, [_P, _P]),
    "pqg_set_inversion": (_I, [_P, _P]),
    "pqg_set_ubg": (_I, [_P, _P]),
    "pqg_set_qy": (_I, [_P, _P]),
    "pqg_set_filter": (_I, [_P, _P]),
    "pqg_set_rek": (_I, [_P, _D]),
    "pqg_set_engine": (_I, [_P, _I]),
    "pqg_get_engine": (_I, [_P]),
    "pqg_rfft2": (_I, [_P, _P, _P, _I, _P]),
    "pqg_irfft2": (_I, [_P, _P, _P, _I, _P]),
    "pqg_invert": (_I, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "pqg_do_advection": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "pqg_do_friction": (_I, [_P, _P, _P, _P]),
    "pqg_do_q_forcing": (_I, [_P, _P, _P, _P, _P]),
    "pqg_do_uv_forcing": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "pqg_forward_timestep": (_I, [_P, _I, _D, _P, _P, _P, _P, _P, _I, _P]),
    "pqg_step": (_I, [_P, ctypes.POINTER(State), _I, ctypes.POINTER(Aux),
                      _P]),
    "pqg_step_profile": (_I, [_P, ctypes.POINTER(State), _I,
                              ctypes.POINTER(_D), ctypes.POINTER(_I), _P]),
    "pqg_rfft2_noalloc": (_I, [_P, _P, _I, _I, _I, _P]),
    "pqg_nonfinite": (_I, [_P, ctypes.POINTER(_I)]),
    "pqg_clear_nonfinite": (_I, [_P]),
    "pqg_ens_last_error": (ctypes.c_char_p, []),
    "pqg_ens_create": (_I, [ctypes.POINTER(_P), _I, _I, _I, _I, _I]),
    "pqg_ens_destroy": (_I, [_P]),
    "pqg_ens_set_constants": (_I, [_P, _P, _P, _P, _P, _D]),
    "pqg_ens_set_members": (_I, [_P, _P, _P, _P]),
    "pqg_ens_set_q": (_I, [_P, _P, _P]),
    "pqg_ens_get_q": (_I, [_P, _P, _P]),
    "pqg_ens_step": (_I, [_P, _I, _P]),
    "pqg_ens_step_many": (_I, [ctypes.POINTER(_P), _I, _I, _P]),
    "pqg_ens_energy": (_I, [_P, _P, _P, _P]),
    "pqg_ens_set_closure": (_I, [_P, _P]),
    "pqg_ens_autotune": (_I, [_P, _P, _P]),
    "pqg_ens_state": (_I, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P),
                           ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_D)]),
    "pqg_advect": (_I, [_P, _P, _P, _P, _I, _P, _P]),
    "pqg_inversion_matrix": (_I, [_I, _I, _I, _I, _P, _P, _P, _P, _P]),
    "pqg_diag_accumulate": (_I, [_P, _I, ctypes.POINTER(DiagFields), _P, _P]),
    "pqg_coarse_forcing": (_I, [_P, _P, _P, _P, _P, _P]),
    "pqg_smag_strain": (_I, [_I, _I, _I, _P, _P, _P, _P, _P, _P]),
    "pqg_smag_stress": (_I, [_I, _I, _I, _P, _D, _P, _P, _P]),
    "pqg_smag_divergence": (_I, [_I, _I, _I, _P, _P, _P, _P, _P]),
    "pqg_zb_gradients": (_I, [_I, _I, _I, _P, _P, _P, _P, _P, _P]),
    "pqg_zb_products": (_I, [_I, _I, _I, _P, _P, _P]),
    "pqg_zb_combine": (_I, [_I, _I, _I, _P, _P, _P, _D, _P, _P]),
    "pqg_lap_power": (_I, [_I, _I, _I, _P, _P, _I, _D, _P, _P, _P]),
    "pqg_layer_mix": (_I, [_I, _I, ctypes.c_longlong, _P, _P, _P, _P]),
    "pqg_mul_scaled": (_I, [ctypes.c_longlong, _P, _D, _P, _P, _P]),
    "pqg_backscatter": (_I, [_I, _I, _I, _P, _P, _P, _P, _D, _D, _P, _P, _P]),
    "pqg_ring_normalize": (_I, [_I, _I, _I, _P, _P, _D, _P, _P, _P]),
    "pqg_cnn_last_error": (ctypes.c_char_p, []),
    "pqg_cnn_create": (_I, [ctypes.POINTER(_P), _I, _P, _I, _I, _I]),
    "pqg_cnn_destroy": (_I, [_P]),
    "pqg_cnn_nparams": (_I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    "pqg_cnn_shape": (_I, [_P] + [ctypes.POINTER(_I)] * 5),
    "pqg_cnn_set_params": (_I, [_P, _P, _P]),
    "pqg_cnn_get_params": (_I, [_P, _P, _P]),
    "pqg_cnn_get_grads": (_I, [_P, _P, _P]),
    "pqg_cnn_set_norm": (_I, [_P, _P, _P, _P, _P]),
    "pqg_cnn_forward": (_I, [_P, _P, _I, _P, _I, _I, _P]),
    "pqg_cnn_backward": (_I, [_P, _P, _P, _I, _P, _P]),
    "pqg_cnn_adam": (_I, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, _P]),
    "pqg_cnn_train_step": (_I, [_P, _P, _P, _I, ctypes.c_float, _P, _P]),
    "pqg_cnn_status": (_I, [_P, _P]),
    "pqg_cnn_set_fault": (_I, [_P, _I, ctypes.c_ulonglong]),
}

_lock = threading.Lock()
_lib = None


class PQGError(RuntimeError):
    """Error status returned by the CUDA library."""

    def __init__(self, code, msg):
        super().__init__("pyqg_gb300 error %d: %s" % (code, msg))
        self.code = code


def load(path=None):
    """Load the shared library and declare every entry point."""
    path = path or lib_path()
    if not os.path.exists(path):
        raise ImportError(
            "pyqg_gb300 CUDA library not built (%s); run "
            "`python -m pyqg_gb300.build`" % path)
    h = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(h, name)
        f.restype = res
        f.argtypes = args
    return h


def lib():
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                _lib = load()
    return _lib


def check(rc):
    """Raise the matching Python exception for a non-zero status."""
    if rc == PQG_OK:
        return
    msg = lib().pqg_last_error().decode(errors="replace")
    if rc == PQG_ERR_INVALID:
        raise ValueError(msg)
    if rc == PQG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == PQG_ERR_NOMEM:
        raise MemoryError(msg)
    raise PQGError(rc, msg)
