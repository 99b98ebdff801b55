"""Host side of the fused stencil kernel (``fsg_stencil`` in include/fsg.h).

One call reads a float32 window once and writes any subset of hillshade,
slope and the four curvature products, each as float32 or as an
int16/uint8 code plane.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Iterable, Optional, Sequence, Tuple

from .. import _arrays
from .. import _native as N
from .._native import Plane, StencilParams, Tile

OUTPUT_INDEX = {
    "hillshade": N.FSG_OUT_HILLSHADE,
    "slope": N.FSG_OUT_SLOPE,
    "curvature_mean": N.FSG_OUT_CURV_MEAN,
    "curvature_gaussian": N.FSG_OUT_CURV_GAUSSIAN,
    "curvature_planform": N.FSG_OUT_CURV_PLANFORM,
    "curvature_profile": N.FSG_OUT_CURV_PROFILE,
    "dx": N.FSG_OUT_DX,
    "dy": N.FSG_OUT_DY,
}


def resolve_scales(pixel_size, pixel_scale_x, pixel_scale_y) -> Tuple[float, float]:
    """``None`` pixel scales fall back to ``pixel_size`` (_nan_utils.py:67-68)."""
    psx = float(pixel_scale_x) if pixel_scale_x is not None else float(pixel_size if pixel_size else 1.0)
    psy = float(pixel_scale_y) if pixel_scale_y is not None else float(pixel_size if pixel_size else 1.0)
    return psx, psy


def make_params(*, azimuth=315.0, altitude=45.0, z_factor=1.0, pixel_size=1.0, nodata=None,
                unit="degree") -> StencilParams:
    if unit not in N.SLOPE_UNITS:
        unit = "radian"  # _impl_slope.py:182-187: any other unit string yields radians
    p = StencilParams()
    p.azimuth = float(azimuth)
    p.altitude = float(altitude)
    p.z_factor = float(1.0 if z_factor is None else z_factor)
    p.pixel_size = float(pixel_size if pixel_size else 1.0)
    p.has_nodata = 0 if nodata is None else 1
    p.nodata = float("nan") if nodata is None else float(nodata)
    p.slope_unit = N.SLOPE_UNITS[unit]
    return p


def make_plane(t, dtype: str = "float32", qp: Optional[dict] = None) -> Plane:
    pl = Plane()
    pl.ptr = int(t.data_ptr())
    pl.ld = int(t.stride(0)) if t.dim() == 2 else int(t.shape[-1])
    pl.dtype = N.DTYPE_CODES[dtype]
    if dtype != "float32":
        if qp is None:
            raise ValueError(f"quantisation parameters are required for {dtype} output")
        pl.q_a = float(qp["a_coef"])
        pl.q_b = float(qp["b_coef"])
        pl.q_min = int(qp["dn_min"])
        pl.q_max = int(qp["dn_max"])
    return pl


def whole_window_tile(h: int, w: int, psx: float, psy: float) -> Tile:
    t = Tile()
    t.win_y0 = t.win_x0 = 0
    t.win_h, t.win_w = h, w
    t.core_y0 = t.core_x0 = 0
    t.core_h, t.core_w = h, w
    t.out_y0 = t.out_x0 = 0
    t.pixel_scale_x, t.pixel_scale_y = psx, psy
    return t


def launch(view: _arrays.DevView, tiles: Sequence[Tile], params: StencilParams,
           planes: Dict[int, Plane], stream: Optional[int] = None) -> None:
    arr = (Plane * N.FSG_STENCIL_NOUT)()
    for idx, pl in planes.items():
        arr[idx] = pl
    tarr = (Tile * max(1, len(tiles)))(*tiles)
    s = _arrays.current_stream_handle() if stream is None else stream
    N.check(N.lib().fsg_stencil(C.c_void_p(view.ptr), view.ld, view.h, view.w, tarr, len(tiles),
                                C.byref(params), arr, C.c_void_p(s)))


def stencil_block(block, outputs: Iterable[str], *, azimuth=315.0, altitude=45.0, z_factor=1.0,
                  pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None, unit="degree",
                  nodata=None, out_dtype: str = "float32", quantize: Optional[Dict[str, dict]] = None):
    """Fused products of one window; returns ``{name: array}`` (same shape as ``block``)."""
    v = _arrays.as_device_f32_2d(block)
    psx, psy = resolve_scales(pixel_size, pixel_scale_x, pixel_scale_y)
    params = make_params(azimuth=azimuth, altitude=altitude, z_factor=z_factor, pixel_size=pixel_size,
                         nodata=nodata, unit=unit)
    res = {}
    planes = {}
    for name in outputs:
        if name not in OUTPUT_INDEX:
            raise ValueError(f"unknown stencil output {name!r}")
        t = _arrays.empty(v.h, v.w, out_dtype, device=v.tensor.device)
        planes[OUTPUT_INDEX[name]] = make_plane(t, out_dtype, (quantize or {}).get(name))
        res[name] = t
    if v.h * v.w == 0:
        return {k: _arrays.wrap_result(t, v.origin) for k, t in res.items()}
    launch(v, [whole_window_tile(v.h, v.w, psx, psy)], params, planes)
    return {k: _arrays.wrap_result(t, v.origin) for k, t in res.items()}


def launch_host(raster_host, tiles: Sequence[Tile], params: StencilParams, planes_host: Dict[int, Plane],
                stream: Optional[int] = None) -> None:
    """``fsg_stencil_host``: raster and output planes in host memory (pinned for overlap)."""
    arr = (Plane * N.FSG_STENCIL_NOUT)()
    for idx, pl in planes_host.items():
        arr[idx] = pl
    tarr = (Tile * max(1, len(tiles)))(*tiles)
    h, w = int(raster_host.shape[0]), int(raster_host.shape[1])
    ld = int(raster_host.stride(0)) if hasattr(raster_host, "stride") else int(raster_host.strides[0] // 4)
    ptr = int(raster_host.data_ptr()) if hasattr(raster_host, "data_ptr") else int(raster_host.ctypes.data)
    s = _arrays.current_stream_handle() if stream is None else stream
    N.check(N.lib().fsg_stencil_host(C.c_void_p(ptr), ld, h, w, tarr, len(tiles), C.byref(params), arr,
                                     C.c_void_p(s)))


def host_plane(t, dtype: str = "float32", qp: Optional[dict] = None) -> Plane:
    """Plane over a host tensor / array (pinned memory recommended)."""
    pl = Plane()
    pl.ptr = int(t.data_ptr()) if hasattr(t, "data_ptr") else int(t.ctypes.data)
    pl.ld = int(t.stride(0)) if hasattr(t, "stride") else int(t.strides[0] // t.itemsize)
    pl.dtype = N.DTYPE_CODES[dtype]
    if dtype != "float32":
        pl.q_a, pl.q_b = float(qp["a_coef"]), float(qp["b_coef"])
        pl.q_min, pl.q_max = int(qp["dn_min"]), int(qp["dn_max"])
    return pl
