"""ctypes binding of libtfv.so (include/tfv.h).

The library is built in-tree by ``torch_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback behind this package.
"""

import ctypes as C
import os
from pathlib import Path

from . import build as _build

TFV_OK, TFV_EINVAL, TFV_ENUMERIC, TFV_ECUDA = 0, 1, 2, 3
TFV_FP64, TFV_FP32 = 0, 1
BC = {"Open": 0, "Reflective": 1, "Periodic": 2, "Inflow": 3}
BC_ALIASES = {"open": 0, "transmissive": 0, "outflow": 0, "reflective": 1, "wall": 1,
              "slip": 1, "periodic": 2, "wrap": 2, "inflow": 3}
LIMITERS = {"VanLeer": 0, "Albada": 1, "MINBEE": 2, "Superbee": 3, "Unos": 4}
MODELS = {"arrhenius": 0, "znd": 1}
CLOSURES = {"si": 0, "nondimensional": 1}
CONTROLLERS = {"Sound Speed Controlled": 0, "w=0": 1}
VARIANTS = {"Variante 1 - Original": 0, "Variante_2": 1}
WAVESPEEDS = {"Pressure Based": 0, "Enthalpy Based": 1}

STATUS = {0: "READY", 1: "DONE", 2: "ERR_MAXSTEPS", 3: "ERR_STALL", 4: "ERR_NONPHYSICAL",
          5: "ERR_REACTIVE", 6: "ERR_SPECIES", 7: "ERR_CHEMISTRY", 8: "RETRY",
          9: "ERR_DEVICE_WAIT"}
READY, DONE, ERR_CHEMISTRY, RETRY, ERR_DEVICE_WAIT = 0, 1, 7, 8, 9
STATUS_MESSAGES = {
    2: "Maximum steps reached before requested final time",
    3: "Integration stalled before requested final time",
    4: "Hydrodynamic update produced a nonphysical state",
    5: "Could not find stable reactive step",
    6: "3D scalar transport left the physical interval",
    7: "Reaction requires a physical state and reactant fractions in [0,1]",
    9: "A device-side wait on a tensor copy timed out",
}


class Config(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("counts", C.c_int32 * 3), ("lengths", C.c_double * 3),
        ("bc", C.c_int32 * 3), ("limiter", C.c_int32), ("gamma", C.c_double),
        ("cfl", C.c_double), ("t_end", C.c_double), ("max_steps", C.c_int64),
        ("reactive", C.c_int32), ("kinetic_model", C.c_int32), ("closure", C.c_int32),
        ("q_heat", C.c_double), ("activation", C.c_double), ("pre_exponential", C.c_double),
        ("inlet_primitive", C.c_double * 4), ("controller", C.c_int32),
        ("variant", C.c_int32), ("wavespeed", C.c_int32), ("spacing", C.c_double * 3),
    ]


class Tile(C.Structure):
    _fields_ = [("tx", C.c_int32), ("ty", C.c_int32), ("chunk", C.c_int32),
                ("persistent_ctas", C.c_int32), ("tma", C.c_int32)]


class Report(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("dt", C.c_double), ("initial_integral", C.c_double * 5),
        ("boundary_integral", C.c_double * 5), ("source_integral", C.c_double * 5),
        ("steps", C.c_int64), ("status", C.c_int32), ("current", C.c_int32),
        ("fallback_steps", C.c_int32), ("last_fallback", C.c_int32),
    ]


GEOMETRIES = {"cartesian": 0, "cylindrical": 1, "annular": 2, "spherical": 3}
FACE_TYPES = {"outflow": 0, "wall": 1, "periodic": 2, "inflow": 3, "pressure_outlet": 4,
              "stagnation_inlet": 5}


class MetricFace(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("has_backflow", C.c_int32), ("primitive", C.c_double * 5),
        ("lambda_", C.c_double), ("beta", C.c_double), ("pressure", C.c_double),
        ("total_pressure", C.c_double), ("total_temperature", C.c_double),
        ("gas_constant", C.c_double),
    ]


class MetricConfig(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("n", C.c_int32 * 3), ("lengths", C.c_double * 3),
        ("geometry", C.c_int32), ("limiter", C.c_int32), ("reactive", C.c_int32),
        ("model", C.c_int32), ("cfl", C.c_double), ("gamma", C.c_double), ("t_end", C.c_double),
        ("max_steps", C.c_int64), ("q", C.c_double), ("ea", C.c_double), ("a", C.c_double),
        ("faces", MetricFace * 6),
    ]


_VP = C.c_void_p
_SIGS = {
    "tfv_metric_factor_count": ([C.POINTER(MetricConfig)], C.c_int64),
    "tfv_metric_create": ([C.c_int32, C.POINTER(MetricConfig), C.POINTER(C.c_double),
                           C.POINTER(_VP)], C.c_int),
    "tfv_metric_workspace_size": ([_VP, C.POINTER(C.c_size_t)], C.c_int),
    "tfv_metric_bind": ([_VP, _VP, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP), _VP], C.c_int),
    "tfv_metric_advance": ([_VP, C.c_int32], C.c_int),
    "tfv_metric_report": ([_VP, C.POINTER(Report)], C.c_int),
    "tfv_metric_integrals": ([_VP, C.POINTER(C.c_double)], C.c_int),
    "tfv_metric_restore": ([_VP, C.POINTER(Report)], C.c_int),
    "tfv_metric_set_current": ([_VP, C.c_int32], C.c_int),
    "tfv_metric_destroy": ([_VP], C.c_int),
    "tfv_rusanov_flux": ([C.c_int32, C.c_int32, C.c_int64, C.c_int32, _VP, _VP, _VP, _VP, _VP,
                          _VP], C.c_int),
    "tfv_version": ([], C.c_char_p),
    "tfv_last_error": ([], C.c_char_p),
    "tfv_batch_create": ([C.c_int32, C.c_int32, C.c_int32, C.POINTER(Config), C.POINTER(Tile),
                          C.POINTER(_VP)], C.c_int),
    "tfv_batch_workspace_size": ([_VP, C.POINTER(C.c_size_t)], C.c_int),
    "tfv_batch_ring_size": ([_VP, C.POINTER(C.c_int32)], C.c_int),
    "tfv_batch_bind": ([_VP, _VP, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP), _VP], C.c_int),
    "tfv_batch_advance": ([_VP, C.c_int32], C.c_int),
    "tfv_batch_use_graph": ([_VP, C.c_int32], C.c_int),
    "tfv_batch_report": ([_VP, C.POINTER(Report)], C.c_int),
    "tfv_batch_integrals": ([_VP, C.POINTER(C.c_double)], C.c_int),
    "tfv_batch_replan": ([_VP], C.c_int),
    "tfv_batch_restore": ([_VP, C.POINTER(Report)], C.c_int),
    "tfv_batch_set_flux_outputs": ([_VP, C.c_int32, _VP, _VP, _VP], C.c_int),
    "tfv_batch_destroy": ([_VP], C.c_int),
    "tfv_batch_profile": ([_VP, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                           C.POINTER(C.c_float)], C.c_int),
    "tfv_hllc_flux": ([C.c_int32, C.c_int32, C.c_int64, _VP, _VP, _VP, _VP, _VP, _VP], C.c_int),
    "tfv_step_workspace_size": ([C.POINTER(Config), C.c_int32, C.POINTER(C.c_size_t)], C.c_int),
    "tfv_hydro_step": ([C.POINTER(Config), C.c_int32, _VP, _VP, _VP, C.c_double, _VP, _VP, _VP,
                        _VP, C.POINTER(C.c_int32), _VP], C.c_int),
    "tfv_hydro_step_static": ([C.POINTER(Config), C.c_int32, _VP, _VP, _VP, C.c_double, _VP, _VP,
                               _VP, C.POINTER(C.c_int32), _VP], C.c_int),
}

_lib = None


def checked():
    """TORCH_GB300_CHECKED=1 selects the checked build of the library."""
    return os.environ.get("TORCH_GB300_CHECKED", "0") not in ("", "0")


def library_path():
    return _build.library(checked())


def load(build_if_missing=True):
    """Load libtfv.so (building it first if needed and a toolkit is present)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if build_if_missing and (not path.exists() or _build._sources_newer(path)):
        _build.build(checked=checked())
    if not path.exists():
        raise RuntimeError(f"libtfv.so is missing at {path}; run python -m torch_gb300.build")
    lib = C.CDLL(os.fspath(path))
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def last_error():
    return load().tfv_last_error().decode()


def check(code, what=""):
    """Map an ABI status to the reference's exception types."""
    if code == TFV_OK:
        return
    msg = last_error() or what
    if code == TFV_EINVAL:
        raise ValueError(msg)
    if code == TFV_ENUMERIC:
        raise RuntimeError(msg)
    raise RuntimeError(f"CUDA error: {msg}")


def bc_code(name):
    try:
        return BC_ALIASES[str(name).lower()]
    except KeyError:
        raise ValueError(f"Unknown boundary: {name}") from None


def ptr(tensor):
    return None if tensor is None else _VP(tensor.data_ptr())


def stream_ptr(stream):
    return _VP(stream.cuda_stream) if stream is not None else None
