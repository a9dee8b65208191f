"""ctypes binding of the C ABI in include/mara_gpu.h.

The library is built in-tree (mara2_gb300/_lib/libmara_gpu.so) by
mara2_gb300/build.py.  There is no fallback: if the library or a CUDA device
is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmara_gpu.so")

LAW = {"hydro": 0, "mhd": 1, "rmhd": 2}
RECON = {"pcm": 0, "plm": 1, "weno5": 2}
RIEMANN = {"hlle": 0, "hllc": 1}
BC = {"periodic": 0, "outflow": 1, "reflecting": 2}
WENO_IS = {"js96": 0, "borges08": 1, "shenzha10": 2}
PRECISION = {"fp64": 0, "mixed": 1, "mixed_fp64": 2}

MARA_OK = 0
MARA_ERR_INVERSION_FAILURE = 16
MARA_ERR_SUPERLUMINAL = 17
MARA_ERR_BAD_EIGENVALUES = 18
MARA_ERR_GUARD_TOO_SMALL = 19
MARA_ERR_CONFIG = 20
MARA_ERR_CUDA = 32
MARA_ERR_NO_DEVICE = 33
MARA_ERR_ARGUMENT = 34
MARA_ERR_TOO_LARGE = 35


class MaraGpuConfig(C.Structure):
    _fields_ = [
        ("law", C.c_int), ("recon", C.c_int), ("riemann", C.c_int), ("bc", C.c_int),
        ("rk_order", C.c_int), ("disable_ct", C.c_int), ("weno_is", C.c_int),
        ("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("ng", C.c_int * 3),
        ("lower", C.c_double * 3), ("upper", C.c_double * 3),
        ("gamma", C.c_double), ("plm_theta", C.c_double), ("shenzha_A", C.c_double),
        ("pressure_floor", C.c_double), ("precision", C.c_int), ("device", C.c_int),
        ("cooling_rate", C.c_double),
    ]


class MaraGpuStats(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("failures", C.c_int), ("first_zone", C.c_int * 3), ("first_code", C.c_int),
        ("steps", C.c_int64), ("kernel_launches", C.c_int64), ("last_dt", C.c_double),
    ]


# Every symbol include/mara_gpu.h declares, with (restype, argtypes).
_D = C.POINTER(C.c_double)
_H = C.c_void_p
class MaraSourceTermsArgs(C.Structure):
    """MaraSourceTermsArgs (include/mara_gpu.h)."""
    _fields_ = [("P", C.c_void_p), ("S", C.c_void_p), ("sP", C.c_longlong), ("N", C.c_int * 3),
                ("ng", C.c_int * 3), ("nq", C.c_int), ("lower", C.c_double * 3), ("dx", C.c_double * 3),
                ("aux", C.c_double * 8), ("stream", C.c_void_p)]


SOURCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(MaraSourceTermsArgs))

MARA_INIT_PLANAR_RIEMANN, MARA_INIT_SHEAR_LAYER, MARA_INIT_CYLINDER = 1, 2, 3


class MaraInitialData(C.Structure):
    """MaraInitialData (include/mara_gpu.h)."""
    _fields_ = [("kind", C.c_int), ("left", C.c_double * 8), ("right", C.c_double * 8), ("x0", C.c_double * 3),
                ("normal", C.c_double * 3), ("radius", C.c_double), ("noise", C.c_double),
                ("seed", C.c_ulonglong)]

SIGNATURES = {
    "mara_gpu_create": (C.c_int, [C.POINTER(MaraGpuConfig), C.POINTER(C.c_void_p)]),
    "mara_gpu_destroy": (C.c_int, [_H]),
    "mara_gpu_upload": (C.c_int, [_H, C.c_void_p]),
    "mara_gpu_download": (C.c_int, [_H, C.c_void_p]),
    "mara_gpu_advance": (C.c_int, [_H, C.c_double, C.c_double]),
    "mara_gpu_advance_host": (C.c_int, [_H, C.c_void_p, C.c_double, C.c_double]),
    "mara_gpu_courant": (C.c_int, [_H, _D]),
    "mara_gpu_run": (C.c_int, [_H, C.c_int, C.c_double, C.c_double, _D, C.POINTER(C.c_int)]),
    "mara_gpu_run_async": (C.c_int, [_H, C.c_int, C.c_double, C.c_double]),
    "mara_gpu_synchronize": (C.c_int, [_H]),
    "mara_gpu_stats": (C.c_int, [_H, C.POINTER(MaraGpuStats)]),
    "mara_gpu_stream": (C.c_void_p, [_H]),
    "mara_gpu_host_register": (C.c_int, [C.c_void_p, C.c_size_t]),
    "mara_gpu_host_unregister": (C.c_int, [C.c_void_p]),
    "mara_gpu_set_kernel_timing": (C.c_int, [_H, C.c_int]),
    "mara_gpu_kernel_times": (C.c_int, [_H, _D, C.POINTER(C.c_int64)]),
    "mara_gpu_device_bytes": (C.c_int64, [_H]),
    "mara_gpu_monopole": (C.c_int, [_H, C.c_double, _D]),
    "mara_gpu_num_diagnostics": (C.c_int, [_H]),
    "mara_gpu_generate": (C.c_int, [_H, C.POINTER(MaraInitialData)]),
    "mara_gpu_set_source_terms": (C.c_int, [_H, C.c_void_p, C.c_void_p]),
    "mara_source_uniform_gravity": (C.c_int, [C.c_void_p, C.POINTER(MaraSourceTermsArgs)]),
    "mara_gpu_volume_diagnostics": (C.c_int, [_H, C.c_void_p, C.POINTER(C.c_int)]),
    "mara_gpu_field_diagnostics": (C.c_int, [_H, C.c_double, C.c_void_p]),
    "mara_gpu_status_string": (C.c_char_p, [C.c_int]),
    "mara_gpu_quartic_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "mara_gpu_ct_monopole": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int]),
    "mara_gpu_ct_current": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_int]),
    "mara_gpu_assign_vector_potential": (C.c_int, [_H, C.c_void_p, C.c_double]),
    "mara_gpu_fp64_peak": (C.c_int, [C.c_int, _D]),
    "mara_gpu_advance_noalloc": (C.c_int, [C.POINTER(MaraGpuConfig), C.c_void_p, C.c_void_p, C.c_double,
                                           C.c_void_p]),
}

_lib = None


def load(path: str | None = None):
    """Load (once) and return the CUDA library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with mara2_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def status_string(code: int) -> str:
    return load().mara_gpu_status_string(code).decode()


class MaraError(RuntimeError):
    def __init__(self, code: int, where: str = ""):
        self.code = code
        super().__init__(f"{where}: status {code} ({status_string(code)})")


def check(code: int, where: str = "") -> None:
    if code != MARA_OK:
        raise MaraError(code, where)


def config_from_scheme(s, precision: str = "fp64", device: int = 0) -> MaraGpuConfig:
    c = MaraGpuConfig()
    c.law, c.recon, c.riemann, c.bc = LAW[s.law], RECON[s.recon], RIEMANN[s.riemann], BC[s.bc]
    c.rk_order, c.disable_ct, c.weno_is = s.rk_order, int(s.disable_ct), WENO_IS[s.weno_is]
    c.ni, c.nj, c.nk = s.shape
    for a in range(3):
        c.ng[a] = s.ng[a]
        c.lower[a], c.upper[a] = s.lower[a], s.upper[a]
    c.gamma, c.plm_theta, c.shenzha_A, c.pressure_floor = s.gamma, s.plm_theta, s.shenzha_A, s.pressure_floor
    c.precision, c.device = PRECISION[precision], device
    c.cooling_rate = s.cooling_rate
    return c
