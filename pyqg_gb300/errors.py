"""Exceptions (same names as ``pyqg/errors.py``)."""


class PYQGError(Exception):
    """Base class for all pyqg exceptions."""


class DiagnosticNotFilledError(PYQGError):
    """A diagnostic was read before any value was accumulated."""

    def __init__(self, dname):
        super().__init__(f"Diagnostic {dname} has not been filled. "
                         "Please adjust tavestart and taveint.")
