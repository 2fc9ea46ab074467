"""The model state and its diagnostics as an xarray Dataset
(``Model.to_dataset``, pyqg/xarray_output.py:118-174).

``model_to_dataset_spec(m)`` builds the dataset as plain numpy data: the
three arguments of ``xarray.Dataset(data_vars, coords=..., attrs=...)``,
each variable and coordinate a ``(dims, values, attrs)`` tuple.  It needs
no xarray.  ``model_to_dataset(m)`` passes them to xarray and raises
``ImportError`` when xarray is missing, as the reference module does when
it is imported.

The layout is pyqg's output format: the variable names, dimension names,
units and long names below (typos included) are the ones the reference
writes, so that files and analysis code written for pyqg read these
datasets unchanged.  Values come from the model's getters, which copy the
device state to the host.
"""
import numpy as np

from .errors import DiagnosticNotFilledError

SPATIAL = ("time", "lev", "y", "x")
SPECTRAL = ("time", "lev", "l", "k")

# state variables: dims
VARIABLE_DIMS = {
    "q": SPATIAL, "u": SPATIAL, "v": SPATIAL, "ufull": SPATIAL, "vfull": SPATIAL,
    "qh": SPECTRAL, "uh": SPECTRAL, "vh": SPECTRAL, "ph": SPECTRAL, "dqhdt": SPECTRAL,
    "Ubg": ("lev",), "Qy": ("lev",),
}


def _attrs(units, long_name):
    return {"units": units, "long_name": long_name}


VARIABLE_ATTRS = {
    "q": _attrs("s^-1", "potential vorticity in real space"),
    "u": _attrs("m s^-1", "zonal velocity anomaly"),
    "v": _attrs("m s^-1", "meridional velocity anomaly"),
    "ufull": _attrs("m s^-1", "zonal full velocities in real space"),
    "vfull": _attrs("m s^-1", "meridional full velocities in real space"),
    "qh": _attrs("s^-1", "potential vorticity in spectral space"),
    "uh": _attrs("m s^-1", "zonal velocity anomaly in spectral space"),
    "vh": _attrs("m s^-1", "meridional velocity anomaly in spectral space"),
    "ph": _attrs("m^2 s^-1", "streamfunction in spectral space"),
    "p": _attrs("m^2 s^-1", "streamfunction in real space"),
    "Ubg": _attrs("m s^-1", "background zonal velocity"),
    "Qy": _attrs("m^-1 s^-1", "background potential vorticity gradient"),
    "dqhdt": _attrs("s^-2", "previous partial derivative of potential vorticity wrt. time in spectral space"),
    "dqdt": _attrs("s^-2", "previous partial derivative of potential vorticity wrt. time in real space"),
}

# spectral variables also written in real space
INVERTED = {"dqhdt": "dqdt", "ph": "p"}

COORD_ATTRS = {
    "time": {"long_name": "model time", "units": "s"},
    "lev": {"long_name": "vertical levels"},
    "lev_mid": {"long_name": "vertical level interface"},
    "x": {"long_name": "real space grid points in the x direction", "units": "grid point"},
    "y": {"long_name": "real space grid points in the y direction", "units": "grid point"},
    "l": {"long_name": "spectal space grid points in the l direction", "units": "meridional wavenumber"},
    "k": {"long_name": "spectal space grid points in the k direction", "units": "zonal wavenumber"},
}

COORD_VALUES = {
    "time": lambda m: np.array([m.t]),
    "lev": lambda m: np.arange(1, m.nz + 1),
    "lev_mid": lambda m: np.arange(1.5, m.nz + .5),
    "x": lambda m: np.asarray(m.x)[0, :],
    "y": lambda m: np.asarray(m.y)[:, 0],
    "l": lambda m: np.asarray(m.ll),
    "k": lambda m: np.asarray(m.kk),
}

# model parameters written as global attributes "pyqg:<name>" (when set)
GLOBAL_ATTRS = ("beta", "delta", "del2", "dt", "filterfac", "L", "M", "nk", "nl", "ntd", "nx", "ny",
                "nz", "pmodes", "radii", "rd", "rho", "rek", "taveint", "tavestart", "tc", "tmax",
                "tsnapint", "tsnapstart", "twrite", "W")

TITLE = "pyqg: Python Quasigeostrophic Model"
REFERENCE = "https://pyqg.readthedocs.io/en/latest/index.html"


def model_to_dataset_spec(m):
    """(data_vars, coords, attrs) of the model's dataset, as numpy data."""
    data_vars = {}
    for name, dims in VARIABLE_DIMS.items():
        if hasattr(m, name):
            data = np.array(getattr(m, name))
            if "time" in dims:
                data = data[np.newaxis, ...]
            data_vars[name] = (dims, data, dict(VARIABLE_ATTRS[name]))
    for spectral, spatial in INVERTED.items():
        if hasattr(m, spectral):
            data = np.asarray(m.ifft(np.asarray(getattr(m, spectral))))
            data_vars[spatial] = (SPATIAL, data[np.newaxis, ...], dict(VARIABLE_ATTRS[spatial]))
    coords = {name: ((name,), np.array(fn(m)), dict(COORD_ATTRS[name])) for name, fn in COORD_VALUES.items()}
    attrs = {}
    for name in GLOBAL_ATTRS:
        if hasattr(m, name):
            attrs["pyqg:" + name] = getattr(m, name)
    for name, entry in m.diagnostics.items():
        try:
            data = m.get_diagnostic(name)
        except DiagnosticNotFilledError:
            continue
        dims = tuple(entry["dims"])
        data = np.asarray(data)
        if data.ndim == 0:
            data = data[np.newaxis]
        dattrs = {"long_name": entry["description"], "units": entry["units"]}
        if "time" not in dims:
            data_vars[name] = (("time",) + dims, data[np.newaxis, ...], dattrs)
        else:
            data_vars[name] = (dims, data, dattrs)
    attrs["title"] = TITLE
    attrs["reference"] = REFERENCE
    return data_vars, coords, attrs


def model_to_dataset(m):
    """The model's state and filled diagnostics as an ``xarray.Dataset``."""
    try:
        import xarray as xr
    except ImportError:
        raise ImportError(
            "Xarray output in Pyqg requires the Xarray package, which is not installed on your "
            "system. Please install Xarray in order to activate this feature.")
    data_vars, coords, attrs = model_to_dataset_spec(m)
    return xr.Dataset(data_vars, coords=coords, attrs=attrs)
