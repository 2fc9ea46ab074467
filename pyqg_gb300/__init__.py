"""pyqg_gb300: pyqg's pseudo-spectral QG models with the time step on a
GB300 GPU (hand-written sm_103a CUDA behind a C ABI).

Drop-in for ``import pyqg``: the model classes, parameterizations and
diagnostic tools have the same names and signatures.
"""
from .errors import PYQGError, DiagnosticNotFilledError
from .kernel import PseudoSpectralKernel
from .model import Model
from .qg_model import QGModel
from .bt_model import BTModel
from .sqg_model import SQGModel
from .layered_model import LayeredModel
from .parameterizations import *  # noqa: F401,F403
from . import diagnostic_tools
from .ensemble import Ensemble

__version__ = "0.1.0"
