"""ctypes binding of libgbdyn.so (include/gbdyn.h).  There is no fallback: without the built
library, or without a CUDA device, every call raises."""

import ctypes
from pathlib import Path

import numpy as np

from .build import LIBGBDYN, LIBGBMATH

GB_OK, GB_ECFL, GB_EHALO, GB_ELEVELS, GB_ESEARCH, GB_EARG, GB_ECUDA, GB_ETIMEOUT = 0, 1, 2, 4, 8, 16, 32, 64
# launch-shape keys of gb_tune_set / gb_tune_get
TUNE_KEYS = {"column_threads": 0, "cell_threads": 1, "lu_warps": 2, "apply_threads": 3, "lu_lanes": 4}


class GBView(ctypes.Structure):
    """gb_view: pointer, extents and element strides of a device array of rank <= 4."""

    _fields_ = [("p", ctypes.c_void_p), ("n", ctypes.c_int64 * 4), ("s", ctypes.c_int64 * 4)]


class CFLError(RuntimeError):
    """A sub-cycle cap was reached (pydyn.kernels.CFLError, kernels.py:60-61)."""


class DeviceError(RuntimeError):
    """A failure reported by the device library."""


_P = ctypes.POINTER(GBView)
_VP = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double

# name -> (restype, argtypes); every entry point include/gbdyn.h declares
SIGNATURES = {
    "gb_create": (_I, [_I, ctypes.POINTER(_VP)]),
    "gb_destroy": (None, [_VP]),
    "gb_last_error": (ctypes.c_char_p, []),
    "gb_alloc": (_I, [_VP, ctypes.c_size_t, ctypes.POINTER(_VP)]),
    "gb_free": (_I, [_VP, _VP]),
    "gb_put": (_I, [_VP, _VP, _VP, ctypes.c_size_t]),
    "gb_get": (_I, [_VP, _VP, _VP, ctypes.c_size_t]),
    "gb_get_async": (_I, [_VP, _VP, _VP, ctypes.c_size_t]),
    "gb_copy_d2d": (_I, [_VP, _VP, _VP, ctypes.c_size_t]),
    "gb_host_alloc": (_I, [ctypes.c_size_t, ctypes.POINTER(_VP)]),
    "gb_host_free": (_I, [_VP]),
    "gb_stream_sync": (_I, [_VP]),
    "gb_sync": (_I, [_VP]),
    "gb_status_peek": (_I, [_VP, ctypes.POINTER(_I)]),
    "gb_launches": (ctypes.c_int64, [_VP]),
    "gb_stream": (_VP, [_VP]),
    "gb_capture_begin": (_I, [_VP]),
    "gb_capture_end": (_I, [_VP, ctypes.POINTER(_VP)]),
    "gb_graph_launch": (_I, [_VP, _VP]),
    "gb_graph_destroy": (_I, [_VP]),
    "gb_event_create": (_I, [ctypes.POINTER(_VP)]),
    "gb_event_record": (_I, [_VP, _VP]),
    "gb_stream_wait": (_I, [_VP, _VP]),
    "gb_work_reserve": (_I, [_VP, ctypes.c_size_t]),
    "gb_stream_priority": (_I, [_VP, _I]),
    "gb_work_size": (ctypes.c_size_t, [_VP]),
    "gb_device_name": (_I, [_VP, ctypes.c_char_p, _I]),
    "gb_tune_set": (_I, [_VP, _I, _I]),
    "gb_tune_get": (_I, [_VP, _I, ctypes.POINTER(_I)]),
    "gb_event_elapsed_ms": (_I, [_VP, _VP, ctypes.POINTER(ctypes.c_float)]),
    "gb_event_sync": (_I, [_VP]),
    "gb_event_destroy": (_I, [_VP]),
    "gb_cfl_reset": (_I, [_VP]),
    "gb_cfl_failed": (_I, [_VP, ctypes.POINTER(_I)]),
    "gb_box": (_I, [_VP, _I, _P, _P, _P, _D, _D]),
    "gb_seqsum": (_I, [_VP, _P, _P, _I, _D]),
    "gb_interp": (_I, [_VP, _P, _P, _P, _VP]),
    "gb_iadd": (_I, [_VP, _VP, _I]),
    "gb_stamp": (_I, [_VP, _VP, _I]),
    "gb_copy_many": (_I, [_VP, _VP, _I, ctypes.c_size_t]),
    "gb_scratch_info": (_I, [_VP, ctypes.POINTER(_VP), ctypes.POINTER(ctypes.c_size_t)]),
    "gb_fill_mass_change": (_I, [_VP, _P, _P, _P, _VP, _VP, _D]),
    "gb_mass_check": (_I, [_VP, _P, _P, _P, _P, _VP, _D, _VP]),
    "gb_balance_fft": (_I, [_VP, _P, _P, _P, _P, _VP, _VP, _VP]),
    "gb_match_sum": (_I, [_VP, _I, _P, _P, _I, _I, _I, _I, _I, _I]),
    "gb_balance_direct": (_I, [_VP, _P, _P, _P, _P, _VP, _VP, _I, _I, _I, _I, _I, _I]),
    "gb_compare": (_I, [_VP, _P, _P, _VP]),
    "gb_advect_x": (_I, [_VP, _P, _P, _P, _P, _P, _P, _VP, _I, _I, _I, _I, _I, _VP, _VP]),
    "gb_advect_y": (_I, [_VP, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _VP]),
    "gb_advect_y_noalloc": (_I, [_VP, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _VP]),
    "gb_advect_z": (_I, [_VP, _P, _P, _P, _P, _P, _P, _I, _I, _VP]),
    "gb_advect_z_scope": (_I, [_VP, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I]),
    "gb_cfl_x": (_I, [_VP, _P, _P, _VP, _I, _I, _I, _I]),
    "gb_cfl_y": (_I, [_VP, _P, _P, _I]),
    "gb_cfl_z": (_I, [_VP, _P, _P, _I, _I, _I, _I, _I]),
    "gb_advect_x_held": (_I, [_VP, _P, _P, _P, _P, _P, _P, _I, _I]),
    "gb_advect_y_held": (_I, [_VP, _P, _P, _P, _P, _P, _P, _P, _I, _VP, _I, _I]),
    "gb_cfl_x_held": (_I, [_VP, _P, _P, _I]),
    "gb_cfl_y_held": (_I, [_VP, _P, _P, _P, _I, _VP, _I]),
    "gb_put_xedges": (_I, [_VP, _P, _P, _I, _I, _I, _I, _I, _I, _I, _D, _D, _I]),
    "gb_put_yedges": (_I, [_VP, _P, _P, _I, _I, _I, _I, _I, _I, _I, _D, _D, _I]),
    "gb_compress_xedges": (_I, [_VP, _P, _I, _I, _I, _I, _I, _I, _I]),
    "gb_compress_yedges": (_I, [_VP, _P, _I, _I, _I, _I, _I, _I, _I]),
    "gb_mix_edges": (_I, [_VP, _P, _I, _I, _I, _I, _I, _I]),
    "gb_update_parent": (_I, [_VP, _P, _P, _I, _I, _I, _I, _I]),
    "gb_coarsen_block": (_I, [_VP, _P, _P, _I, _I, _I, _I, _I, _D]),
    "gb_coarsen_ambm": (_I, [_VP, _P, _P, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I, _I]),
    "gb_convec": (_I, [_VP, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _VP, _VP, ctypes.c_int64, ctypes.c_int64, _VP, _I,
                       _D, _I, _VP, _VP, _VP, _VP]),
    "gb_calc_kzz": (_I, [_VP, _P, _P, _P, _P, _P, _P, _P, _VP, _VP, _VP, _I, _D, _D, _D, _P, _P]),
    "gb_loss_rates": (_I, [_VP, _P, _P, _VP, _P, _P, _P, _P, _P, _P, _P, _P, _VP, _D, _D, _D, _D, _D, _P, _P]),
    "gb_chemistry": (_I, [_VP, _P, _P, _VP, _P, _P, _P, _P, _P, _P, _P, _P, _VP, _D, _D, _D, _D, _D, _VP, _I,
                          ctypes.c_uint32, _P, _P, _P, _P, _P, _VP, _VP]),
    "gb_chem_krates": (_I, [_VP, _P, _VP, _I, _P]),
    "gb_sources": (_I, [_VP, _P, _P, _P, _VP, _D, _I, _I, _VP, _I]),
    "gb_math_eval":(_I, [_VP, _I, _VP, _VP, _VP, ctypes.c_int64]),
    "gb_advect_z_last": (_I, [_VP, _VP]),
    "gb_adjoint_x": (_I, [_VP, _P, _P, _P, _P, _P, _P, _VP, _I]),
    "gb_adjoint_y": (_I, [_VP, _P, _P, _P, _P, _P, _P, _VP]),
    "gb_adjoint_z": (_I, [_VP, _P, _P, _P, _P, _P, _P, _VP]),
    "gb_adjoint_convec": (_I, [_VP, _P, _P, _P, _P, _VP, _VP, _I, _I]),
    "gb_adjoint_sources": (_I, [_VP, _P, _P, _P, _VP, _D, _I, _VP, _I]),
    "gb_fp64_rate": (_I, [_VP, _I, ctypes.POINTER(_D)]),
    "gb_fluxes_from_meteo": (_I, [_VP, _P, _P, _VP, _D, _P, _P, _P]),
    "gb_m2phlb": (_I, [_VP, _P, _P, _P, _VP, _VP, _VP, _I, _I, _I, _VP]),
}

_LIB = []


def lib():
    """The loaded libgbdyn.so with its prototypes set; raises if it was not built."""
    if not _LIB:
        path = Path(LIBGBDYN)
        if not path.exists():
            raise RuntimeError(f"pydyn_gb300: {path} is not built (run pydyn_gb300.build.build())")
        L = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _LIB.append(L)
    return _LIB[0]


def last_error():
    msg = lib().gb_last_error()
    return msg.decode() if msg else ""


def check(rc, what=""):
    """Raise for a non-zero status of a host-side call."""
    if rc == GB_OK:
        return
    if rc & GB_ECFL:
        raise CFLError(f"{what}: {last_error()}")
    if rc & (GB_EHALO | GB_ELEVELS):
        raise ValueError(f"{what}: {last_error()}")
    raise DeviceError(f"{what} failed ({rc}): {last_error()}")


_MATH = []


def mathlib():
    """libgbmath.so: the host build of the device's transcendental functions."""
    if not _MATH:
        path = Path(LIBGBMATH)
        if not path.exists():
            raise RuntimeError(f"pydyn_gb300: {path} is not built")
        L = ctypes.CDLL(str(path))
        for name, nargs in (("exp", 1), ("log", 1), ("pow", 2), ("cos", 1), ("sin", 1)):
            f = getattr(L, name)
            f.restype, f.argtypes = ctypes.c_double, [ctypes.c_double] * nargs
        _MATH.append(L)
    return _MATH[0]


def host_math(name, *arrays):
    """Apply libgbmath's `name` elementwise on the host (float64 arrays, broadcast)."""
    f = getattr(mathlib(), name)
    arrs = np.broadcast_arrays(*(np.asarray(a, dtype=np.float64) for a in arrays))
    out = np.empty(arrs[0].shape)
    flat = [a.ravel() for a in arrs]
    o = out.ravel()
    for k in range(o.size):
        o[k] = f(*(float(a[k]) for a in flat))
    return out
