"""ctypes binding of libfsg.so (the C ABI declared in include/fsg.h).

The library is loaded from ``fujishadergpu_gb300/lib/libfsg.so``.  There is no
CPU fallback: if the library is missing or no CUDA device is present every
entry point raises, so a run that "works" is always the CUDA path.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_LIB_PATH = os.environ.get("FSG_LIBRARY") or os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib",
                                                          "libfsg.so")
_lock = threading.Lock()
_lib = None

# ----------------------------------------------------------------- constants
FSG_OK = 0
FSG_ERR_INVALID = -1
FSG_ERR_SHAPE = -2
FSG_ERR_DTYPE = -3
FSG_ERR_CUDA = -4
FSG_ERR_TIMEOUT = -5
FSG_ERR_ABORTED = -6
FSG_ERR_WORKSPACE = -7
FSG_ERR_UNSUPPORTED = -8

FSG_F32, FSG_U8, FSG_I16 = 0, 1, 2
DTYPE_CODES = {"float32": FSG_F32, "uint8": FSG_U8, "int16": FSG_I16}

FSG_OUT_HILLSHADE = 0
FSG_OUT_SLOPE = 1
FSG_OUT_CURV_MEAN = 2
FSG_OUT_CURV_GAUSSIAN = 3
FSG_OUT_CURV_PLANFORM = 4
FSG_OUT_CURV_PROFILE = 5
FSG_OUT_DX = 6
FSG_OUT_DY = 7
FSG_STENCIL_NOUT = 8
CURVATURE_OUT = {"mean": FSG_OUT_CURV_MEAN, "gaussian": FSG_OUT_CURV_GAUSSIAN,
                 "planform": FSG_OUT_CURV_PLANFORM, "profile": FSG_OUT_CURV_PROFILE}
SLOPE_UNITS = {"degree": 0, "percent": 1, "radian": 2}


class FsgError(RuntimeError):
    """A libfsg.so call failed; ``code`` is the FSG_ERR_* status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"libfsg error {code}: {message}")
        self.code = code


class FsgValueError(FsgError, ValueError):
    """Invalid argument / shape: the reference raises ValueError in these cases."""


# ------------------------------------------------------------------- structs
class Plane(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("ld", C.c_int64), ("dtype", C.c_int32), ("reserved", C.c_int32),
                ("q_a", C.c_float), ("q_b", C.c_float), ("q_min", C.c_int32), ("q_max", C.c_int32)]


class Tile(C.Structure):
    _fields_ = [("win_y0", C.c_int32), ("win_x0", C.c_int32), ("win_h", C.c_int32), ("win_w", C.c_int32),
                ("core_y0", C.c_int32), ("core_x0", C.c_int32), ("core_h", C.c_int32), ("core_w", C.c_int32),
                ("out_y0", C.c_int32), ("out_x0", C.c_int32), ("reserved0", C.c_int32), ("reserved1", C.c_int32),
                ("pixel_scale_x", C.c_double), ("pixel_scale_y", C.c_double)]


class StencilParams(C.Structure):
    _fields_ = [("azimuth", C.c_double), ("altitude", C.c_double), ("z_factor", C.c_double),
                ("pixel_size", C.c_double), ("nodata", C.c_double), ("has_nodata", C.c_int32),
                ("slope_unit", C.c_int32)]


class TopoUSMParams(C.Structure):
    _fields_ = [("radii", C.POINTER(C.c_int32)), ("weights", C.POINTER(C.c_double)), ("nradii", C.c_int32),
                ("has_nodata", C.c_int32), ("pixel_size", C.c_double), ("nodata", C.c_double),
                ("coarse_dev", C.c_void_p), ("coarse_ld", C.c_int64), ("coarse_h", C.c_int32),
                ("coarse_w", C.c_int32), ("full_h", C.c_int64), ("full_w", C.c_int64), ("w_large", C.c_double),
                ("scale", C.c_double), ("path", C.c_int32)]


TOPOUSM_PATHS = {"exact": 0, "tensor": 1}


class StoreFinish(C.Structure):
    _fields_ = [("divisor", C.c_float), ("stretch_lo", C.c_float), ("stretch_scale", C.c_float),
                ("keep_nodata_values", C.c_int32)]


COMBINE_WSUM, COMBINE_MAX, COMBINE_MIN = 0, 1, 2


class AoParams(C.Structure):
    _fields_ = [("num_samples", C.c_int32), ("has_nodata", C.c_int32), ("radius", C.c_double),
                ("intensity", C.c_double), ("pixel_size", C.c_double), ("nodata", C.c_double),
                ("stretch_lo", C.c_double), ("stretch_scale", C.c_double)]


class OpennessParams(C.Structure):
    _fields_ = [("openness_type", C.c_int32), ("num_directions", C.c_int32), ("max_distance", C.c_int32),
                ("mode", C.c_int32), ("pixel_size", C.c_double), ("nodata", C.c_double),
                ("has_nodata", C.c_int32), ("reserved", C.c_int32), ("stretch_lo", C.c_double),
                ("stretch_scale", C.c_double)]


# Exported symbols and their signatures (kept in sync with include/fsg.h).
_SIGNATURES = {
    "fsg_abi_version": (C.c_int, []),
    "fsg_version": (C.c_char_p, []),
    "fsg_last_error": (C.c_char_p, []),
    "fsg_launch_count": (C.c_int64, []),
    "fsg_timing_begin": (C.c_int, [C.c_int32]),
    "fsg_timing_end": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "fsg_kernel_errors": (C.c_int, [C.POINTER(C.c_uint32)]),
    "fsg_scratch_high_water": (C.c_int, [C.POINTER(C.c_uint64), C.c_int32]),
    "fsg_nodata_mask": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                  C.c_void_p, C.c_int64, C.c_void_p]),
    "fsg_stencil": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile), C.c_int32,
                              C.POINTER(StencilParams), C.POINTER(Plane), C.c_void_p]),
    "fsg_stencil_plan": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile), C.c_int32,
                                   C.POINTER(StencilParams), C.POINTER(Plane), C.POINTER(C.c_void_p)]),
    "fsg_plan_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fsg_plan_destroy": (None, [C.c_void_p]),
    "fsg_stencil_host": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile), C.c_int32,
                                   C.POINTER(StencilParams), C.POINTER(Plane), C.c_void_p]),
    "fsg_topousm": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile), C.c_int32,
                              C.POINTER(TopoUSMParams), C.POINTER(Plane), C.c_void_p]),
    "fsg_topousm_plan": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile), C.c_int32,
                                   C.POINTER(TopoUSMParams), C.POINTER(Plane), C.POINTER(C.c_void_p)]),
    "fsg_topousm_coarse_field": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                           C.POINTER(C.c_double), C.c_int32, C.c_double, C.c_void_p, C.c_int64,
                                           C.c_void_p]),
    "fsg_overview": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.c_void_p,
                               C.c_int32, C.c_int32, C.c_int64, C.c_void_p]),
    "fsg_topousm_downsample_factor": (C.c_int, [C.c_double, C.c_double]),
    "fsg_percentile": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_double), C.c_int32,
                                 C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_void_p]),
    "fsg_std": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.c_void_p]),
    "fsg_key_histogram": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_uint32, C.c_uint32, C.c_int32,
                                    C.c_int32, C.POINTER(C.c_uint64), C.c_void_p]),
    "fsg_percentile_noalloc": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_double), C.c_int32,
                                         C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_void_p]),
    "fsg_openness": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile), C.c_int32,
                               C.POINTER(OpennessParams), C.POINTER(Plane), C.c_void_p, C.c_int64, C.c_void_p]),
    "fsg_openness_plan": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile), C.c_int32,
                                    C.POINTER(OpennessParams), C.POINTER(Plane), C.c_void_p, C.c_int64,
                                    C.POINTER(C.c_void_p)]),
    "fsg_ambient_occlusion": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile), C.c_int32,
                                        C.POINTER(AoParams), C.POINTER(Plane), C.c_void_p]),
    "fsg_ambient_occlusion_plan": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Tile),
                                             C.c_int32, C.POINTER(AoParams), C.POINTER(Plane),
                                             C.POINTER(C.c_void_p)]),
    "fsg_nearest_sample": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                     C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]),
    "fsg_coarse_average": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                     C.POINTER(C.c_double), C.c_int32, C.c_void_p, C.c_int64, C.c_void_p,
                                     C.c_int64, C.POINTER(C.c_int32), C.c_void_p]),
    "fsg_value_mode": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, C.c_double,
                                 C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_void_p]),
    "fsg_count_equal": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_double, C.POINTER(C.c_int64),
                                  C.c_void_p]),
    "fsg_pushpull_fill": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p,
                                    C.c_int64, C.c_void_p]),
    "fsg_edge_connected": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                     C.c_void_p]),
    "fsg_fill_apply": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                 C.c_int32, C.POINTER(C.c_double), C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                 C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                 C.POINTER(C.c_int32), C.c_void_p]),
    "fsg_openness_offsets": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32]),
    "fsg_affine": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32,
                             C.POINTER(Plane), C.c_void_p]),
    "fsg_smooth": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double,
                             C.c_void_p, C.c_int64, C.c_void_p]),
    "fsg_pad_reflect": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                  C.c_int32, C.c_int32, C.c_double, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]),
    "fsg_accumulate": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_float, C.c_int32, C.c_void_p,
                                 C.c_int64, C.c_void_p]),
    "fsg_sample_coarse_accumulate": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                               C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                               C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_int32,
                                               C.c_float, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]),
    "fsg_combine": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_int32,
                              C.c_void_p, C.c_int64, C.c_void_p]),
    "fsg_masked_store": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                   C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_int32, C.POINTER(StoreFinish),
                                   C.POINTER(Plane), C.c_void_p]),
    "fsg_downsample_nan_aware": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                           C.c_int64, C.c_void_p]),
    "fsg_upsample_to_shape": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                        C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                        C.c_void_p]),
    "fsg_conv_pack_weights": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "fsg_conv3x3": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                              C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fsg_conv3x3_wgrad": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "fsg_head_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float, C.c_int64, C.c_void_p, C.c_void_p]),
    "fsg_head_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
}


def library_path() -> str:
    return _LIB_PATH


def lib():
    """Load libfsg.so once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                raise FsgError(FSG_ERR_UNSUPPORTED,
                               f"{_LIB_PATH} is missing: build it with "
                               "`python -m fujishadergpu_gb300.build` (needs nvcc)")
            L = C.CDLL(_LIB_PATH)
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def exported_symbols():
    return list(_SIGNATURES)


def check(status: int) -> None:
    if status == FSG_OK:
        return
    msg = lib().fsg_last_error().decode("utf-8", "replace")
    if status in (FSG_ERR_INVALID, FSG_ERR_SHAPE, FSG_ERR_DTYPE):
        raise FsgValueError(status, msg)
    raise FsgError(status, msg)


def launch_count() -> int:
    return int(lib().fsg_launch_count())


def kernel_errors() -> int:
    """Device-side failure flags since the last call (cleared on read; 0 = none)."""
    v = C.c_uint32(0)
    check(lib().fsg_kernel_errors(C.byref(v)))
    return int(v.value)


class kernel_timer:
    """Context manager timing the dominant kernel of each library call (CUDA events
    recorded by the library around those launches); ``.ms`` = summed kernel time,
    ``.launches`` = number of timed launches."""

    def __init__(self, max_launches: int = 4096):
        self.max_launches = int(max_launches)
        self.ms = 0.0
        self.launches = 0

    def __enter__(self):
        check(lib().fsg_timing_begin(self.max_launches))
        return self

    def __exit__(self, *exc):
        tot, n = C.c_double(0.0), C.c_int32(0)
        check(lib().fsg_timing_end(C.byref(tot), C.byref(n)))
        self.ms, self.launches = float(tot.value), int(n.value)
        return False
