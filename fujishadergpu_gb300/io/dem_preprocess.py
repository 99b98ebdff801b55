"""NoData detection and void fill before the hot path (io/dem_preprocess.py of
the reference, ``preprocess_dem_to_cog`` :462-726, on an in-memory raster).

The reference converts a GDAL raster to a COG and, on the way, (1) reads a
nearest-resampled coarse sample, (2) detects undeclared NoData sentinels on it
(a dominant sentinel / range extreme, a dominant constant border), (3) builds
the NaN-aware coarse average, (4) fills its voids with a push-pull pyramid and,
for ``fill_mode='enclosed'``, marks the border-connected voids as exterior, and
(5) streams the raster in row bands, setting NoData to NaN and filling the
allowed voids from the bilinear coarse surface.  Here the raster is a device
array and the file I/O is left out; (1), (3), (4) and (5) are CUDA kernels
(``fsg_nearest_sample``, ``fsg_coarse_average``, ``fsg_pushpull_fill``,
``fsg_edge_connected``, ``fsg_fill_apply``); for (2) the exact value counts
come from the device (``fsg_value_mode``, ``fsg_count_equal``) and only the
decisions and the few thousand ring values are handled on the host.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

from .. import _arrays
from .. import _native as N

FILL_MODES = ("none", "enclosed", "all")
FILL_CODES = {"none": 0, "enclosed": 1, "all": 2}

# Common undeclared NoData fills (io/dem_preprocess.py:228-238).
NODATA_SENTINELS = (
    0.0, -9999.0, -99999.0, 9999.0,
    -32768.0, 32767.0, -32767.0, 65535.0,
    -2147483648.0, 2147483647.0, -2147483647.0,
    -128.0, 127.0, 255.0,
)


def coarse_shape(width: int, height: int, coarse_max: int) -> Tuple[int, int]:
    """_coarse_shape (:278-282) -> (ch, cw)."""
    scale = max(width / coarse_max, height / coarse_max, 1.0)
    return max(1, int(round(height / scale))), max(1, int(round(width / scale)))


def coarse_oversample(ch: int, cw: int, k: int = 4, max_intermediate: int = 4096) -> int:
    """The oversampling of the nearest coarse read (:537-539, :156-158)."""
    k = max(2, int(k))
    while k > 2 and max(ch * k, cw * k) > int(max_intermediate):
        k -= 1
    return k


def _known_or_extreme(cand: float, vmin: float, vmax: float) -> bool:
    known = any(abs(cand - s) <= 1e-6 * max(1.0, abs(s)) for s in NODATA_SENTINELS)
    return known or abs(cand) >= 1e30 or cand == vmin or cand == vmax


def _sentinel_rule(sample, declared, min_fraction: float, stream) -> Optional[float]:
    """The sentinel rule of _detect_sentinel_nodata (io/dem_preprocess.py:241-275) on the
    device sample: the value statistics come from fsg_value_mode (exact counts), the
    decision is the reference's."""
    h, w = sample.shape
    nf, lo, hi, mv, mc = C.c_int64(), C.c_double(), C.c_double(), C.c_double(), C.c_int64()
    N.check(N.lib().fsg_value_mode(C.c_void_p(sample.data_ptr()), w, h, w, C.c_void_p(declared.data_ptr()), w,
                                   float(min_fraction), C.byref(nf), C.byref(lo), C.byref(hi), C.byref(mv),
                                   C.byref(mc), stream))
    if nf.value < 64 or mc.value == 0 or mc.value / float(nf.value) < float(min_fraction):
        return None
    cand = float(mv.value)
    return cand if _known_or_extreme(cand, float(lo.value), float(hi.value)) else None


def _border_rule(sample, declared, min_border_fraction: float, stream, min_total_fraction: float = 0.02):
    """The border rule of _detect_border_nodata (io/dem_preprocess.py:191-225) with the
    outer ring on the host and the whole-sample count of the candidate from fsg_count_equal."""
    h, w = sample.shape
    if h < 8 or w < 8:
        return None
    parts = [(sample[0, :], declared[0, :]), (sample[-1, :], declared[-1, :]),
             (sample[1:-1, 0], declared[1:-1, 0]), (sample[1:-1, -1], declared[1:-1, -1])]
    ring = np.concatenate([p.cpu().numpy() for p, _ in parts])
    ok = np.concatenate([(d.cpu().numpy() == 0) for _, d in parts])
    ring = ring[ok & np.isfinite(ring)]
    if ring.size == 0:
        return None
    vals, counts = np.unique(ring, return_counts=True)
    i = int(np.argmax(counts))
    cand = float(vals[i])
    if counts[i] / ring.size < float(min_border_fraction):
        return None
    cnt = C.c_int64()
    N.check(N.lib().fsg_count_equal(C.c_void_p(sample.data_ptr()), w, h, w, cand, C.byref(cnt), stream))
    if cnt.value / float(h * w) < float(min_total_fraction):
        return None
    return cand


@dataclass
class PrepareResult:
    array: object                        # the normalised / filled raster (device, float32)
    extra_nodata: List[float]            # override + detected sentinels treated as NoData
    coarse_shape: Tuple[int, int]
    oversample: int
    do_fill: bool
    surface: Optional[object] = None     # the coarse fill surface (device)
    exterior: Optional[object] = None    # the coarse exterior mask (device, uint8)
    extras: dict = field(default_factory=dict)


def _doubles(vals):
    arr = (C.c_double * max(1, len(vals)))(*[float(v) for v in vals])
    return arr, len(vals)


def prepare_dem(dem, *, nodata: Optional[float] = None, fill_mode: str = "enclosed", coarse_max: int = 2048,
                nodata_override: Optional[float] = None, detect_nodata: bool = True,
                nodata_border_fraction: float = 0.5, nodata_sentinel_fraction: float = 0.05,
                out=None) -> PrepareResult:
    """preprocess_dem_to_cog's NoData handling and fill on a device raster.

    ``nodata``: the raster's declared NoData (None: none; NaN allowed).  ``out``: a
    float32 device array of the raster's shape to write into (may be ``dem`` itself);
    default a new array.  Raises ValueError for an unknown fill mode and RuntimeError
    when ``fill_mode='all'`` leaves a non-finite cell (:815-822)."""
    fill_mode = str(fill_mode).lower()
    if fill_mode not in FILL_MODES:
        raise ValueError(f"Unknown fill_mode={fill_mode!r}. Choose from {FILL_MODES}.")
    torch = _arrays._torch()
    v = _arrays.as_device_f32_2d(dem, name="dem")
    H, W = v.h, v.w
    dev = v.tensor.device
    lib = N.lib()
    stream = C.c_void_p(_arrays.current_stream_handle())
    has_nd = 0 if nodata is None else 1
    ndv = float("nan") if nodata is None else float(nodata)
    ch, cw = coarse_shape(W, H, int(coarse_max))
    extra: List[float] = []
    if nodata_override is not None and math.isfinite(float(nodata_override)):
        extra.append(float(nodata_override))
    k = coarse_oversample(ch, cw)
    sample = torch.empty((ch * k, cw * k), device=dev, dtype=torch.float32)
    declared = torch.empty((ch * k, cw * k), device=dev, dtype=torch.uint8)
    N.check(lib.fsg_nearest_sample(C.c_void_p(v.ptr), v.ld, H, W, ch * k, cw * k, ndv, has_nd,
                                   C.c_void_p(sample.data_ptr()), cw * k, C.c_void_p(declared.data_ptr()), cw * k,
                                   stream))
    if detect_nodata:
        for det in (_sentinel_rule(sample, declared, nodata_sentinel_fraction, stream),
                    _border_rule(sample, declared, nodata_border_fraction, stream)):
            if det is None:
                continue
            already = any(np.isclose(det, x) for x in extra)
            decl = nodata is not None and bool(np.isclose(det, float(nodata)))
            if not already and not decl:
                extra.append(float(det))
    cvals = list(extra)
    if nodata is not None and math.isfinite(float(nodata)):
        cvals.append(float(nodata))
    coarse = torch.empty((ch, cw), device=dev, dtype=torch.float32)
    valid = torch.empty((ch, cw), device=dev, dtype=torch.uint8)
    arr, n = _doubles(cvals)
    any_void = C.c_int32(0)
    N.check(lib.fsg_coarse_average(C.c_void_p(sample.data_ptr()), cw * k, C.c_void_p(declared.data_ptr()), cw * k,
                                   ch, cw, k, arr, n, C.c_void_p(coarse.data_ptr()), cw,
                                   C.c_void_p(valid.data_ptr()), cw, C.byref(any_void), stream))
    del sample, declared
    do_fill = fill_mode != "none" and bool(any_void.value)
    surface = exterior = None
    if do_fill:
        surface = torch.empty((ch, cw), device=dev, dtype=torch.float32)
        N.check(lib.fsg_pushpull_fill(C.c_void_p(coarse.data_ptr()), cw, C.c_void_p(valid.data_ptr()), cw, ch, cw,
                                      C.c_void_p(surface.data_ptr()), cw, stream))
        if fill_mode == "enclosed":
            exterior = torch.empty((ch, cw), device=dev, dtype=torch.uint8)
            N.check(lib.fsg_edge_connected(C.c_void_p(valid.data_ptr()), cw, ch, cw, 1,   # the voids: valid == 0
                                           C.c_void_p(exterior.data_ptr()), cw, stream))
    if out is None:
        out_t = torch.empty((H, W), device=dev, dtype=torch.float32)
        ov = _arrays.as_device_f32_2d(out_t)
    else:
        ov = _arrays.as_device_f32_2d(out, name="out")
        if (ov.h, ov.w) != (H, W):
            raise ValueError(f"out has shape {(ov.h, ov.w)}, the raster {(H, W)}")
    ex, ne = _doubles(extra)
    nonfinite = C.c_int32(0)
    N.check(lib.fsg_fill_apply(C.c_void_p(v.ptr), v.ld, H, W, 0, H, ndv, has_nd, ex, ne,
                               FILL_CODES[fill_mode] if do_fill else 0,
                               C.c_void_p(surface.data_ptr() if surface is not None else 0), cw,
                               C.c_void_p(exterior.data_ptr() if exterior is not None else 0), cw, ch, cw,
                               C.c_void_p(ov.ptr), ov.ld, C.byref(nonfinite) if fill_mode == "all" else None,
                               stream))
    if fill_mode == "all" and nonfinite.value:
        raise RuntimeError("fill_mode='all' left non-finite pixels")
    return PrepareResult(_arrays.wrap_result(ov.tensor, v.origin), extra, (ch, cw), k, do_fill, surface, exterior,
                         {"coarse": coarse, "valid": valid})


__all__ = ["prepare_dem", "PrepareResult", "FILL_MODES", "coarse_shape", "coarse_oversample"]
