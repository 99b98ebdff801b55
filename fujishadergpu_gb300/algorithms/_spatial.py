"""Spatial (multi-radius) mode of the stencil products.

Reference behaviour, per product (hillshade, slope, curvature):

* ``_smooth_for_radius`` (algorithms/_nan_utils.py:527-552) -> ``fsg_smooth``;
  ``compute_hillshade_spatial_block`` (_impl_hillshade.py:57-67),
  ``compute_slope_spatial_block`` (_impl_slope.py:38-45) and curvature's
  ``_curv_spatial`` (_impl_curvature.py:72-78) smooth, then run the product.
* The local multi-radius branch of ``_direct_hillshade``
  (algorithms/tile/dask_bridge.py:72-108, ``_combine_direct`` :28-69): the
  spatial block per radius on the whole window, float32-normalised weights.
* ``mode='spatial'`` on the tile backend: ``_process_direct`` falls back to
  the product's Dask ``process`` on the tile window as one chunk
  (dask_bridge.py:334-346, :387-403), i.e. ``multiscale_response_fields``
  (_nan_utils.py:441-524): a radius above the window's large-radius threshold
  (``large_radius_threshold``, :219-228) is the product of the whole overview
  (radius and pixel scales divided / multiplied by its decimation) sampled at
  the window's global pixel centres and NaN at NoData (:366-395); the others
  are ``map_overlap(spatial_block, depth, boundary='reflect')``.  The
  responses are combined with the product's weights (_impl_hillshade.py:113-128;
  ``_combine_multiscale_dask`` :182-213) and the tile processor restores NaN at
  the NoData footprint of the core (core/tile_processor.py:973-980).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .. import _arrays
from .. import _native as N
from . import _stencil as S

ALGO_FACTOR = {"hillshade": 1.0, "slope": 1.0, "curvature": 1.1}   # _nan_utils.py:571-581
PRODUCTS = tuple(ALGO_FACTOR)


def smooth_for_radius(block, radius, *, pixel_size: float = 1.0, algorithm_name: str = "default"):
    """``_smooth_for_radius`` on one device block (fsg_smooth)."""
    v = _arrays.as_device_f32_2d(block)
    out = _arrays.empty(v.h, v.w, device=v.tensor.device)
    _smooth_into(v.ptr, v.ld, v.h, v.w, radius, pixel_size, algorithm_name, out)
    return _arrays.wrap_result(out, v.origin)


def _algo_factor(name: str) -> float:
    from .._native import lib  # noqa: F401  (loads the library: fail loudly without it)
    return {"topousm_fast": 1.15, "hillshade": 1.0, "slope": 1.0, "specular": 1.4,
            "atmospheric_scattering": 1.05, "curvature": 1.1, "ambient_occlusion": 1.5,
            "openness": 1.4, "multi_light_uncertainty": 1.25}.get(str(name), 1.0)


def _smooth_into(ptr, ld, h, w, radius, pixel_size, algorithm_name, out, stream=None):
    s = _arrays.current_stream_handle() if stream is None else stream
    N.check(N.lib().fsg_smooth(C.c_void_p(ptr), int(ld), int(h), int(w), float(radius),
                               float(pixel_size if pixel_size else 1.0), _algo_factor(algorithm_name),
                               C.c_void_p(out.data_ptr()), int(out.stride(0)), C.c_void_p(s)))


# --------------------------------------------------------------- products
def _outputs(product: str, kw: dict) -> str:
    if product == "curvature":
        ct = kw.get("curvature_type", "mean")
        return "curvature_" + (ct if ct in ("mean", "gaussian", "planform") else "profile")
    return product


def _stencil_params(product: str, kw: dict, pixel_size: float):
    return S.make_params(azimuth=kw.get("azimuth", 315.0), altitude=kw.get("altitude", 45.0),
                         z_factor=1.0 if kw.get("z_factor") is None else kw.get("z_factor", 1.0),
                         pixel_size=pixel_size, unit=kw.get("unit", "degree"))


def _run_product(src_ptr, src_ld, src_h, src_w, core, product, kw, pixel_size, psx, psy, out_tensor):
    """The product of the (smoothed) array ``src`` with the window = all of src and the
    given core (y0, x0, h, w), written into out_tensor (h x w, float32)."""
    t = N.Tile()
    t.win_y0, t.win_x0, t.win_h, t.win_w = 0, 0, src_h, src_w
    t.core_y0, t.core_x0, t.core_h, t.core_w = core
    t.out_y0, t.out_x0 = 0, 0
    t.pixel_scale_x, t.pixel_scale_y = float(psx), float(psy)
    arr = (N.Plane * N.FSG_STENCIL_NOUT)()
    arr[S.OUTPUT_INDEX[_outputs(product, kw)]] = S.make_plane(out_tensor)
    tiles = (N.Tile * 1)(t)
    p = _stencil_params(product, kw, pixel_size)
    N.check(N.lib().fsg_stencil(C.c_void_p(src_ptr), int(src_ld), int(src_h), int(src_w), tiles, 1, C.byref(p),
                                arr, C.c_void_p(_arrays.current_stream_handle())))


def spatial_block(block, product: str, radius, *, pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None, **kw):
    """The spatial block function of ``product`` (smoothing, then the product)."""
    v = _arrays.as_device_f32_2d(block)
    sm = _arrays.empty(v.h, v.w, device=v.tensor.device)
    _smooth_into(v.ptr, v.ld, v.h, v.w, radius, pixel_size, product, sm)
    out = _arrays.empty(v.h, v.w, device=v.tensor.device)
    psx, psy = S.resolve_scales(pixel_size, pixel_scale_x, pixel_scale_y)
    if v.h * v.w:
        _run_product(sm.data_ptr(), sm.stride(0), v.h, v.w, (0, 0, v.h, v.w), product, kw, pixel_size, psx, psy,
                     out)
    return _arrays.wrap_result(out, v.origin)


def compute_hillshade_spatial_block(block, *, azimuth=315, altitude=45, z_factor=1.0, pixel_size=1.0,
                                    pixel_scale_x=None, pixel_scale_y=None, radius=4.0):
    """_impl_hillshade.py:57-67."""
    return spatial_block(block, "hillshade", radius, pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                         pixel_scale_y=pixel_scale_y, azimuth=azimuth, altitude=altitude, z_factor=z_factor)


def compute_slope_spatial_block(block, *, unit="degree", pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None,
                                radius=4.0):
    """_impl_slope.py:38-45."""
    return spatial_block(block, "slope", radius, pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                         pixel_scale_y=pixel_scale_y, unit=unit)


def compute_curvature_spatial_block(block, *, curvature_type="mean", pixel_size=1.0, pixel_scale_x=None,
                                    pixel_scale_y=None, radius=4.0):
    """curvature's _curv_spatial (_impl_curvature.py:72-78)."""
    return spatial_block(block, "curvature", radius, pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                         pixel_scale_y=pixel_scale_y, curvature_type=curvature_type)


# ------------------------------------------------------------ weights
def clean_normalized_weights(weights) -> Optional[List[float]]:
    """_clean_normalized_weights (_nan_utils.py:142-154)."""
    out = []
    for w in weights:
        try:
            fv = float(w)
        except (TypeError, ValueError):
            return None
        out.append(fv if math.isfinite(fv) and fv > 0 else 0.0)
    s = float(sum(out))
    if s <= 0:
        return None
    return [v / s for v in out]


def combine_weights(weights, n: int, product: str) -> List[float]:
    """The float32 weight of each response.

    hillshade (_impl_hillshade.py:113-123) normalises float32 weights in float32;
    slope / curvature (_combine_multiscale_dask, _nan_utils.py:203-208)
    L1-normalise in float64 (cast to float32 by the multiply).  Weights of the
    wrong length or without a positive sum fall back to the plain mean, taken
    here as weights 1/n.
    """
    if weights is not None and not isinstance(weights, (str, bytes)) and len(weights) == n:
        if product == "hillshade":
            w = np.asarray(weights, dtype=np.float32)
            if np.isfinite(w).all() and float(w.sum()) > 0:
                w = w / w.sum()
                return [float(np.float32(x)) for x in w]
        else:
            c = clean_normalized_weights(weights)
            if c is not None:
                return [float(np.float32(x)) for x in c]
    return [float(np.float32(1.0 / n))] * n


def spatial_depth(product: str, radius) -> int:
    """depth_for_scale (_impl_hillshade.py:98, _impl_slope.py:62, _impl_curvature.py:85)."""
    r = float(radius)
    return max(3, int(r * 2 + 2)) if product == "curvature" else max(2, int(r * 2 + 1))


def large_radius_threshold(win_h: int, win_w: int) -> int:
    """large_radius_threshold of a one-chunk window (_nan_utils.py:219-228)."""
    return int(max(256, int(min(win_h, win_w)) // 16))


# ------------------------------------------------------------ tile loop
class Overview:
    """The unified overview coarse source (read_overview_coarse_dem,
    _nan_utils.py:836-871; tile injection core/tile_processor.py:1529-1546): a
    NaN-aware block-mean overview of at most 2048 px per side, its decimation, and
    the coarse product responses per (radius, pixel scales)."""

    def __init__(self, raster: _arrays.DevView, *, nodata=None, sample_max: int = 2048):
        H, W = raster.h, raster.w
        scale = max(W / sample_max, H / sample_max, 1.0)
        self.ow, self.oh = max(1, int(round(W / scale))), max(1, int(round(H / scale)))
        self.decimation = 0.5 * (W / float(self.ow) + H / float(self.oh))
        self.full = (H, W)
        from ._impl_topousm_fast import overview as _ov
        self.dem = _ov(raster.tensor, (self.oh, self.ow), nodata=nodata)
        self._resp: Dict[tuple, object] = {}

    def response(self, product: str, radius, kw: dict, pixel_size: float, psx: float, psy: float):
        key = (product, float(radius), float(psx), float(psy), tuple(sorted(kw.items())))
        if key not in self._resp:
            fac = float(self.decimation)
            rc = max(1, int(round(float(radius) / fac)))
            self._resp[key] = _arrays.as_device_f32_2d(
                spatial_block(self.dem, product, rc, pixel_size=pixel_size * fac, pixel_scale_x=psx * fac,
                              pixel_scale_y=psy * fac, **kw))
        return self._resp[key]


def spatial_tile(raster: _arrays.DevView, win: Tuple[int, int, int, int], core: Tuple[int, int, int, int],
                 product: str, radii: Sequence[float], weights: Sequence[float], kw: dict, *, pixel_size: float,
                 psx: float, psy: float, nodata, overview: Optional[Overview], plane: N.Plane,
                 scratch: dict, global_offset: Tuple[int, int] = (0, 0)) -> None:
    """One tile of the spatial product: window (y0, x0, h, w) and core (y0, x0, h, w) in
    raster coordinates; the combined core is stored into ``plane`` (addressing the core's
    first pixel).  ``global_offset`` is added to raster coordinates to give the global
    pixel coordinates the overview is sampled at."""
    torch = _arrays._torch()
    lib = N.lib()
    stream = C.c_void_p(_arrays.current_stream_handle())
    wy, wx, wh, ww = win
    cy, cx, ch, cw = core
    has_nd = 0 if nodata is None else 1
    ndv = float("nan") if nodata is None else float(nodata)
    thr = large_radius_threshold(wh, ww)
    dev = raster.tensor.device

    def buf(name, n):
        b = scratch.get(name)
        if b is None or b.numel() < n:
            b = torch.empty(int(n * 1.05) + 1024, device=dev, dtype=torch.float32)
            scratch[name] = b
        return b

    acc = buf("acc", ch * cw)[: ch * cw].view(ch, cw)
    resp = buf("resp", ch * cw)[: ch * cw].view(ch, cw)
    ws = combine_weights(weights, len(radii), product)
    for i, (r, w) in enumerate(zip(radii, ws)):
        first = 1 if i == 0 else 0
        if int(round(float(r))) > thr and overview is not None:
            cr = overview.response(product, r, kw, pixel_size, psx, psy)
            N.check(lib.fsg_sample_coarse_accumulate(
                C.c_void_p(cr.ptr), cr.ld, cr.h, cr.w, C.c_void_p(raster.ptr), raster.ld, raster.h, raster.w,
                cy, cx, ch, cw, cy + int(global_offset[0]), cx + int(global_offset[1]), overview.full[0],
                overview.full[1], ndv, has_nd, C.c_float(w), first, C.c_void_p(acc.data_ptr()), acc.stride(0),
                stream))
            continue
        d = max(1, min(spatial_depth(product, r), min(wh, ww) - 1))
        ph, pw = wh + 2 * d, ww + 2 * d
        padded = buf("pad", ph * pw)[: ph * pw].view(ph, pw)
        smooth = buf("smooth", ph * pw)[: ph * pw].view(ph, pw)
        N.check(lib.fsg_pad_reflect(C.c_void_p(raster.ptr), raster.ld, raster.h, raster.w, wy, wx, wh, ww, d, ndv,
                                    has_nd, C.c_void_p(padded.data_ptr()), pw, stream))
        _smooth_into(padded.data_ptr(), pw, ph, pw, r, pixel_size, product, smooth)
        _run_product(smooth.data_ptr(), pw, ph, pw, (d + cy - wy, d + cx - wx, ch, cw), product, kw, pixel_size,
                     psx, psy, resp)
        N.check(lib.fsg_accumulate(C.c_void_p(resp.data_ptr()), cw, ch, cw, C.c_float(w), first,
                                   C.c_void_p(acc.data_ptr()), cw, stream))
    N.check(lib.fsg_masked_store(C.c_void_p(acc.data_ptr()), cw, C.c_void_p(raster.ptr), raster.ld, raster.h,
                                 raster.w, cy, cx, ch, cw, ndv, has_nd, C.byref(plane), stream))


def spatial_stencil(name: str, dem_gpu, params: dict):
    """``process(dem, mode='spatial' | multi-radius)`` of a stencil product on one window.

    With ``mode='spatial'`` this is the tile backend's Dask fallback on the window as
    one chunk (large radii from ``_overview_coarse_dem`` when the params carry it,
    with ``_tile_origin`` / ``_tile_full_shape``); otherwise the local multi-radius
    branch of ``_direct_hillshade``.
    """
    from ..common.spatial_mode import resolve_spatial_radii_weights
    p = dict(params)
    v = _arrays.as_device_f32_2d(dem_gpu)
    px = float(p.get("pixel_size", 1.0) or 1.0)
    psx, psy = S.resolve_scales(px, p.get("pixel_scale_x"), p.get("pixel_scale_y"))
    kw = _product_kwargs(name, p)
    mode = str(p.get("mode", "local")).lower()
    out = _arrays.empty(v.h, v.w, device=v.tensor.device)
    if v.h * v.w == 0:
        return _arrays.wrap_result(out, v.origin)
    if mode != "spatial":
        # _direct_hillshade local multi-radius branch
        radii = p.get("radii") or [1]
        radii = [max(1.0, float(r)) for r in radii]
        ws = combine_weights(p.get("weights"), len(radii), "hillshade")
        acc = _arrays.empty(v.h, v.w, device=v.tensor.device)
        for i, (r, w) in enumerate(zip(radii, ws)):
            resp = _arrays.as_device_f32_2d(spatial_block(v.tensor, name, r, pixel_size=px, pixel_scale_x=psx,
                                                          pixel_scale_y=psy, **kw))
            if len(radii) == 1:
                return _arrays.wrap_result(resp.tensor, v.origin)
            N.check(N.lib().fsg_accumulate(C.c_void_p(resp.ptr), resp.ld, v.h, v.w, C.c_float(w), 1 if i == 0 else 0,
                                           C.c_void_p(acc.data_ptr()), acc.stride(0),
                                           C.c_void_p(_arrays.current_stream_handle())))
        return _arrays.wrap_result(acc, v.origin)
    radii, weights = resolve_spatial_radii_weights(p.get("radii"), p.get("weights"), px)
    if name == "hillshade" and p.get("weights") is not None:
        weights = p.get("weights")   # _impl_hillshade.py:84-87 keeps the caller's weights
    overview = None
    cdem = p.get("_overview_coarse_dem")
    if cdem is not None and p.get("_overview_decimation") is not None and p.get("_tile_origin") is not None:
        overview = _GivenOverview(cdem, float(p["_overview_decimation"]), p.get("_tile_full_shape") or (v.h, v.w))
    origin = p.get("_tile_origin") or (0, 0)
    plane = S.make_plane(out)
    spatial_tile(v, (0, 0, v.h, v.w), (0, 0, v.h, v.w), name, radii, weights, kw, pixel_size=px, psx=psx, psy=psy,
                 nodata=None, overview=overview, plane=plane, scratch={},
                 global_offset=(int(origin[0]), int(origin[1])))
    return _arrays.wrap_result(out, v.origin)


def _product_kwargs(name: str, p: dict) -> dict:
    if name == "hillshade":
        return {"azimuth": float(p.get("azimuth", 315.0)), "altitude": float(p.get("altitude", 45.0)),
                "z_factor": 1.0 if p.get("z_factor") is None else float(p.get("z_factor", 1.0))}
    if name == "slope":
        return {"unit": str(p.get("unit", "degree"))}
    return {"curvature_type": str(p.get("curvature_type", "mean"))}


class _GivenOverview(Overview):
    """An overview handed in by the caller (``_overview_coarse_dem``)."""

    def __init__(self, coarse_dem, decimation: float, full_shape):
        self.dem = _arrays.as_device_f32_2d(coarse_dem).tensor
        self.oh, self.ow = int(self.dem.shape[0]), int(self.dem.shape[1])
        self.decimation = float(decimation)
        self.full = (int(full_shape[0]), int(full_shape[1]))
        self._resp = {}
