"""Openness (algorithms/_impl_openness.py of the reference).

``compute_openness_vectorized`` keeps the reference signature; ``sampling``
selects the reference's 10 sampled distances per ray ("reference") or every
pixel step ("dense", the exact ray-march the CNN surrogate is trained on).
``compute_openness_raw_degrees`` returns the directional mean angle in
degrees (the quantity the 0.01 degree parity gate and the surrogate's 2
degree MAE gate are stated on).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

from .. import _arrays
from .. import _native as N
from ._base import TileAlgorithm
from ._stencil import make_plane, resolve_scales
from ._stats import robust_unsigned_stretch_stat_func

SAMPLING = {"reference": 0, "dense": 1}


def make_params(*, openness_type="positive", num_directions=16, max_distance=50, pixel_size=1.0,
                sampling="reference", nodata=None, stretch=None) -> N.OpennessParams:
    p = N.OpennessParams()
    p.openness_type = 0 if openness_type == "positive" else 1
    p.num_directions = int(num_directions)
    p.max_distance = int(max_distance)
    p.mode = SAMPLING[sampling]
    p.pixel_size = float(pixel_size if pixel_size else 1.0)
    p.has_nodata = 0 if nodata is None else 1
    p.nodata = float("nan") if nodata is None else float(nodata)
    if stretch is not None and len(stretch) >= 2 and float(stretch[1]) > 1e-12:
        p.stretch_lo, p.stretch_scale = float(stretch[0]), float(stretch[1])
    return p


def run_openness(view, tiles, params, display_plane=None, raw=None, stream=None):
    tarr = (N.Tile * max(1, len(tiles)))(*tiles)
    s = _arrays.current_stream_handle() if stream is None else stream
    N.check(N.lib().fsg_openness(C.c_void_p(view.ptr), view.ld, view.h, view.w, tarr, len(tiles), C.byref(params),
                                 C.byref(display_plane) if display_plane is not None else None,
                                 C.c_void_p(raw.data_ptr() if raw is not None else 0),
                                 int(raw.stride(0)) if raw is not None else 0, C.c_void_p(s)))


def _whole(v, psx, psy):
    t = N.Tile()
    t.win_y0, t.win_x0, t.win_h, t.win_w = 0, 0, v.h, v.w
    t.core_y0, t.core_x0, t.core_h, t.core_w = 0, 0, v.h, v.w
    t.out_y0, t.out_x0 = 0, 0
    t.pixel_scale_x, t.pixel_scale_y = psx, psy
    return t


def _scales(pixel_size, pixel_scale_x, pixel_scale_y):
    # _impl_openness.py:70-71: |pixel_scale| or pixel_size
    sx = abs(float(pixel_scale_x)) if pixel_scale_x is not None else float(pixel_size)
    sy = abs(float(pixel_scale_y)) if pixel_scale_y is not None else float(pixel_size)
    return sx, sy


def openness_planes(block, *, openness_type="positive", num_directions=16, max_distance=50, pixel_size=1.0,
                    pixel_scale_x=None, pixel_scale_y=None, sampling="reference", display=True, raw=False,
                    stretch=None, out_dtype="float32", qp=None, nodata=None):
    v = _arrays.as_device_f32_2d(block)
    sx, sy = _scales(pixel_size, pixel_scale_x, pixel_scale_y)
    params = make_params(openness_type=openness_type, num_directions=num_directions, max_distance=max_distance,
                         pixel_size=pixel_size, sampling=sampling, stretch=stretch, nodata=nodata)
    disp = _arrays.empty(v.h, v.w, out_dtype, device=v.tensor.device) if display else None
    rawt = _arrays.empty(v.h, v.w, device=v.tensor.device) if raw else None
    if v.h * v.w:
        run_openness(v, [_whole(v, sx, sy)], params, make_plane(disp, out_dtype, qp) if display else None, rawt)
    return disp, rawt, v


def compute_openness_vectorized(block, *, openness_type: str = "positive", num_directions: int = 16,
                                max_distance: int = 50, pixel_size: float = 1.0, pixel_scale_x: float = None,
                                pixel_scale_y: float = None, sampling: str = "reference"):
    """Display openness in [0, 1] (_impl_openness.py:31-132)."""
    disp, _, v = openness_planes(block, openness_type=openness_type, num_directions=num_directions,
                                 max_distance=max_distance, pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                                 pixel_scale_y=pixel_scale_y, sampling=sampling)
    return _arrays.wrap_result(disp, v.origin)


def compute_openness_raw_degrees(block, *, openness_type="positive", num_directions=16, max_distance=50,
                                 pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None, sampling="reference",
                                 nodata=None):
    """Directional mean zenith (positive) / nadir (negative) angle in degrees (``nodata``: a
    numeric sentinel treated as NoData, as the tile processor's mask)."""
    _, raw, v = openness_planes(block, openness_type=openness_type, num_directions=num_directions,
                                max_distance=max_distance, pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                                pixel_scale_y=pixel_scale_y, sampling=sampling, display=False, raw=True,
                                nodata=nodata)
    return _arrays.wrap_result(raw, v.origin)


class OpennessAlgorithm(TileAlgorithm):
    """Tile adapter: algorithms/tile/openness.py -> dask_bridge._direct_openness (:208-222)."""

    def process(self, dem_gpu, **params):
        p = self._merged(params)
        if str(p.get("mode", "local")).lower() == "spatial":
            from ._spatial import spatial_openness
            return spatial_openness(dem_gpu, p)
        disp, _, v = openness_planes(
            dem_gpu, openness_type=p.get("openness_type", "positive"), num_directions=p.get("num_directions", 16),
            max_distance=p.get("max_distance", 50), pixel_size=p.get("pixel_size", 1.0),
            pixel_scale_x=p.get("pixel_scale_x"), pixel_scale_y=p.get("pixel_scale_y"),
            sampling=p.get("sampling", "reference"), stretch=p.get("global_stats"))
        return _arrays.wrap_result(disp, v.origin)

    def get_default_params(self) -> dict:
        return {"openness_type": "positive", "num_directions": 16, "max_distance": 50, "pixel_size": 1.0,
                "mode": "local", "radii": None, "weights": None}


__all__ = ["compute_openness_vectorized", "compute_openness_raw_degrees", "OpennessAlgorithm",
           "robust_unsigned_stretch_stat_func"]
