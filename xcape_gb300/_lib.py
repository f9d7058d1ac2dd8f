"""ctypes binding of libxcape_gb300.so (declared in include/xcape_gb300.h).

The library is the only compute path of this package: if it cannot be built
or loaded, every call raises -- there is no CPU fallback.
"""
import ctypes
import os
import threading

from . import _build

XC_OK = 0
XC_ERR_INVALID = 1
XC_ERR_CUDA = 2
XC_ERR_NOMEM = 3
XC_ERR_NODEVICE = 4

XC_F32 = 0
XC_F64 = 1

XC_GUESS_PLAIN = 0
XC_GUESS_LEARNED = 1
XC_GUESS_EXTRAPOLATED = 2
XC_GUESS_SECANT = 3
XC_GUESS_LEARNED_EVERY = 4
XC_GUESS_LEARNED_WARP = 5
XC_GUESS_NPARAM = 4481
XC_MAX_LEVELS = 4096
XC_NOALLOC_MAX_COLUMNS = 1048576
XC_RETRY_FP64 = 256

COL_NOCONV = 1
COL_BADSTART = 2
COL_TOOMANYSTEPS = 4
COL_FP64 = 8

GRID_SIGMA = 1
GRID_PRESSURE_1D = 2
GRID_PRESSURE_3D = 3

_lock = threading.Lock()
_lib = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float
_d = ctypes.c_double

# name -> argtypes (restype is int for all compute entry points)
SIGNATURES = {
    "xc_loopcape_ml": [_vp] * 6 + [_i, _f, _i, _f, _i, _i, _i] + [_vp] * 5 + [_vp],
    "xc_loopcape_pl1d": [_vp] * 6 + [_i, _f, _i, _f, _i, _vp, _i, _i] + [_vp] * 5 + [_vp],
    "xc_loopcape_pl": [_vp] * 6 + [_i, _f, _i, _f, _i, _vp, _i, _i] + [_vp] * 5 + [_vp],
    "xc_loopcape_ex": [_i] + [_vp] * 6 + [_i, _f, _i, _f, _i, _vp, _i, _i, _i] + [_vp] * 6
    + [_vp, ctypes.c_size_t, _vp],
    "xc_loopcape_diag": [_i] + [_vp] * 6 + [_i, _f, _i, _f, _i, _vp, _i, _i, _i] + [_vp] * 6
    + [_vp],
    "xc_loopcape_ex_host": [_i] + [_vp] * 6 + [_i, _f, _i, _f, _i, _vp, _i, _i, _i] + [_vp] * 5
    + [_vp],
    "xc_loopcape_multi_host": [_i] + [_vp] * 6 + [_i, _f, _i, _vp, _f, _i, _vp, _i, _i, _i]
    + [_vp] * 5 + [_vp],
    "xc_loopcape_multi": [_i] + [_vp] * 6 + [_i, _f, _i, _vp, _f, _i, _vp, _i, _i, _i] + [_vp] * 6
    + [_vp, ctypes.c_size_t, _vp],
    "xc_loopcape_ex_noalloc": [_i] + [_vp] * 6 + [_i, _f, _i, _f, _i, _vp, _i, _i, _i]
    + [_vp] * 6 + [_vp],
    "xc_calc_srh": [_i] + [_vp] * 10 + [_i, _vp, _d, _d, _i, _i] + [_vp] * 5 + [_vp],
    "xc_calc_srh_ex": [_i] + [_vp] * 10 + [_i, _vp, _d, _d, _i, _i, _i] + [_vp] * 5 + [_vp],
    "xc_calc_srh_host": [_i] + [_vp] * 10 + [_i, _vp, _d, _d, _i, _i, _i] + [_vp] * 5 + [_vp],
    "xc_cape_srh": [_i] + [_vp] * 10 + [_i, _f, _i, _f, _i, _vp, _d, _d, _i, _i, _i, _i]
    + [_vp] * 10 + [_vp, ctypes.c_size_t, _vp],
    "xc_loop_stdheight_ml": [_vp] * 7 + [_i, _i, _vp, _vp, _vp],
    "xc_loop_stdheight_pl1d": [_vp] * 7 + [_vp, _i, _i, _vp, _vp, _vp],
    "xc_loop_stdheight_pl": [_vp] * 7 + [_vp, _i, _i, _vp, _vp, _vp],
    "xc_bunkers_loop_ml": [_vp] * 6 + [_i, _i, _vp, _vp, _vp, _vp],
    "xc_bunkers_loop_pl": [_vp] * 6 + [_vp, _i, _i, _vp, _vp, _vp, _vp],
    "xc_loop_sreh_ml": [_vp] * 10 + [_d, _i, _i, _vp, _vp, _vp],
    "xc_loop_sreh_pl": [_vp] * 10 + [_d, _vp, _i, _i, _vp, _vp, _vp],
    "xc_pres_lev_pos": [_vp, _vp, _i, _i, _i, _vp, _vp],
    "xc_guess_set_weights": [_vp, _i, _vp],
    "xc_guess_pairs": [ctypes.c_longlong, ctypes.c_ulonglong, _vp, _vp, _vp, _vp],
    "xc_guess_grad": [_vp, _vp, _vp, ctypes.c_longlong, _vp, _vp, _vp],
    "xc_guess_grad_tc": [_vp, _vp, _vp, ctypes.c_longlong, _vp, _vp, _vp, _vp],
    "xc_guess_adam": [_vp, _vp, _vp, _vp, _f, _i, _vp],
    "xc_guess_eval": [_vp, _vp, ctypes.c_longlong, _vp, _vp],
    "xc_release_workspace": [],
    "xc_measure_pipe_peaks": [_vp, _vp, _vp],
    "xc_batch_create": [_i, ctypes.c_longlong, _i, ctypes.POINTER(_vp)],
    "xc_batch_run": [_vp, _vp, _i, _vp],
    "xc_batch_work": [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "xc_batch_destroy": [_vp],
    "xc_copy_list": [_i, _vp, _vp, _vp, _vp],
}

XC_BATCH_MAX_REQUESTS = 65536


class CapeRequest(ctypes.Structure):
    """xc_cape_request (include/xcape_gb300.h): one request of a batch."""
    _fields_ = [("grid", _i), ("nk", _i), ("n2", ctypes.c_longlong), ("ld", ctypes.c_longlong),
                ("p", _vp), ("t3d", _vp), ("td3d", _vp), ("ps", _vp), ("ts", _vp), ("tds", _vp),
                ("pinc", _f), ("source", _i), ("ml_depth", _f), ("adiabat", _i),
                ("cape", _vp), ("cin", _vp), ("mulvl", _vp), ("z_out", _vp), ("status", _vp)]


class XcapeError(RuntimeError):
    """Raised when a library call returns a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"[xcape_gb300 status {code}] {msg}")
        self.code = code


def lib():
    """Load (building first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if _build.needs_build():
                try:
                    _build.build()
                except Exception as exc:  # pragma: no cover - depends on toolchain
                    raise ImportError(
                        "xcape_gb300: the CUDA extension libxcape_gb300.so is missing and could "
                        f"not be built ({exc}); there is no CPU fallback") from exc
            L = ctypes.CDLL(path)
            for name, argtypes in SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = argtypes
                fn.restype = ctypes.c_int
            L.xc_loopcape_workspace_bytes.restype = ctypes.c_size_t
            L.xc_loopcape_workspace_bytes.argtypes = [_i]
            L.xc_last_error.restype = ctypes.c_char_p
            L.xc_last_error.argtypes = []
            L.xc_version.restype = ctypes.c_char_p
            L.xc_version.argtypes = []
            L.xc_alloc_count.restype = ctypes.c_longlong
            L.xc_alloc_count.argtypes = []
            _lib = L
    return _lib


def check(rc):
    if rc != XC_OK:
        raise XcapeError(rc, lib().xc_last_error().decode(errors="replace"))


def call(name, *args):
    check(getattr(lib(), name)(*args))


def version():
    return lib().xc_version().decode()


def exported_symbols():
    """Names of the entry points declared in include/xcape_gb300.h."""
    return sorted(list(SIGNATURES) + ["xc_last_error", "xc_version",
                                      "xc_loopcape_workspace_bytes", "xc_alloc_count"])


def workspace_bytes(n2):
    """Device scratch that lets xc_loopcape_ex order n2 columns."""
    return int(lib().xc_loopcape_workspace_bytes(int(n2)))
