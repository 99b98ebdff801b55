"""Spatial (multi-radius) mode of the stencil products, openness and ambient occlusion.

Reference behaviour, per product (hillshade, slope, curvature, openness,
ambient occlusion):

* ``_smooth_for_radius`` (algorithms/_nan_utils.py:527-552) -> ``fsg_smooth``;
  ``compute_hillshade_spatial_block`` (_impl_hillshade.py:57-67),
  ``compute_slope_spatial_block`` (_impl_slope.py:38-45) and curvature's
  ``_curv_spatial`` (_impl_curvature.py:72-78) smooth, then run the product.
* ``compute_openness_spatial_block`` (_impl_openness.py:135-164): openness
  of the NaN-aware f x f decimation (``fsg_downsample_nan_aware``) with the
  distance divided and the pixel scales multiplied by f, zoomed back to the
  block (``fsg_upsample_to_shape``, evaluated only over the window's core).
* ``compute_ambient_occlusion_spatial_block`` (_impl_ambient_occlusion.py:124-157):
  the same, with the radius divided by f (at least 1, not rounded).
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
  responses are combined as the product's ``agg`` says (_impl_hillshade.py:109-131;
  ``_combine_multiscale_dask`` :182-213), openness is display-stretched with the
  global statistics (_impl_openness.py:216) and the tile processor restores NaN
  at the NoData footprint of the core (core/tile_processor.py:973-980).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .. import _arrays
from .. import _native as N
from . import _stencil as S

ALGO_FACTOR = {"hillshade": 1.0, "slope": 1.0, "curvature": 1.1, "openness": 1.4,   # _nan_utils.py:571-581
               "ambient_occlusion": 1.5}
RAY_PRODUCTS = ("openness", "ambient_occlusion")
PRODUCTS = tuple(ALGO_FACTOR)
STENCIL_PRODUCTS = ("hillshade", "slope", "curvature")


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


def downsample_factor(radius, pixel_size=1.0, algorithm_name="default", base_radius=24.0, max_factor=16) -> int:
    """``_radius_to_downsample_factor`` (_nan_utils.py:555-601): a power of two from the radius,
    the algorithm's factor and the resolution (the block shape does not enter)."""
    r = max(1.0, float(radius))
    px = max(1e-3, float(pixel_size) if pixel_size else 1.0)
    score = (r / max(1.0, base_radius)) * _algo_factor(algorithm_name) * 1.0 * (max(1.0, 1.0 / px) ** 0.35)
    if score <= 1.0:
        return 1
    return int(max(1, min(2 ** int(math.floor(math.log2(score))), max_factor)))


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


def _openness_spatial_into(src_ptr, src_ld, src_h, src_w, core, max_distance, kw, pixel_size, psx, psy, out,
                           buf=None):
    """compute_openness_spatial_block (_impl_openness.py:135-164) of the array ``src``,
    evaluated over ``core`` (y0, x0, h, w) of it into ``out`` (h x w, float32).

    Factor 1: the openness kernel with the window = all of src.  Factor f > 1: the
    f x f NaN-aware decimation, openness there with max(2, round(md / f)) and the
    pixel scales x f, then the NaN-aware zoom back to src's shape over the core only.
    """
    from ._impl_openness import make_params, run_openness
    from ._stencil import make_plane
    torch = _arrays._torch()
    lib = N.lib()
    stream = C.c_void_p(_arrays.current_stream_handle())
    f = downsample_factor(float(max_distance), pixel_size, "openness")
    sx, sy = abs(float(psx)), abs(float(psy))
    if buf is None:
        def buf(name, n):
            return torch.empty(int(n), device=out.device, dtype=torch.float32)
    if f <= 1:
        view = _arrays.DevView(None, int(src_ptr), int(src_h), int(src_w), int(src_ld), "torch")
        t = N.Tile()
        t.win_y0, t.win_x0, t.win_h, t.win_w = 0, 0, src_h, src_w
        t.core_y0, t.core_x0, t.core_h, t.core_w = core
        t.out_y0, t.out_x0 = 0, 0
        t.pixel_scale_x, t.pixel_scale_y = sx, sy
        p = make_params(openness_type=kw.get("openness_type", "positive"),
                        num_directions=kw.get("num_directions", 16), max_distance=int(max_distance),
                        pixel_size=pixel_size)
        run_openness(view, [t], p, make_plane(out))
        return
    hs, ws = (src_h + f - 1) // f, (src_w + f - 1) // f
    small = buf("os_small", hs * ws)[: hs * ws].view(hs, ws)
    N.check(lib.fsg_downsample_nan_aware(C.c_void_p(src_ptr), int(src_ld), int(src_h), int(src_w), int(f),
                                         C.c_void_p(small.data_ptr()), ws, stream))
    rsmall = buf("os_resp", hs * ws)[: hs * ws].view(hs, ws)
    sview = _arrays.DevView(small, small.data_ptr(), hs, ws, ws, "torch")
    md = max(2, int(round(float(max_distance) / float(f))))
    p = make_params(openness_type=kw.get("openness_type", "positive"), num_directions=kw.get("num_directions", 16),
                    max_distance=md, pixel_size=float(pixel_size) * f)
    t = N.Tile()
    t.win_y0, t.win_x0, t.win_h, t.win_w = 0, 0, hs, ws
    t.core_y0, t.core_x0, t.core_h, t.core_w = 0, 0, hs, ws
    t.out_y0, t.out_x0 = 0, 0
    t.pixel_scale_x, t.pixel_scale_y = sx * f, sy * f
    run_openness(sview, [t], p, make_plane(rsmall))
    N.check(lib.fsg_upsample_to_shape(C.c_void_p(rsmall.data_ptr()), ws, hs, ws, int(src_h), int(src_w),
                                      int(core[0]), int(core[1]), int(core[2]), int(core[3]),
                                      C.c_void_p(out.data_ptr()), int(out.stride(0)), stream))


def _ao_spatial_into(src_ptr, src_ld, src_h, src_w, core, radius, kw, pixel_size, psx, psy, out, buf=None):
    """compute_ambient_occlusion_spatial_block (_impl_ambient_occlusion.py:124-157) of the
    array ``src``, evaluated over ``core`` (y0, x0, h, w) of it into ``out`` (h x w, float32).

    Factor 1: the AO kernel with the window = all of src.  Factor f > 1: the f x f NaN-aware
    decimation, AO there with the radius max(1, r / f) and the pixel scales x f, then the
    NaN-aware zoom back to src's shape over the core only.
    """
    from ._impl_ambient_occlusion import make_params, run_ambient_occlusion, whole_tile
    from ._stencil import make_plane
    torch = _arrays._torch()
    lib = N.lib()
    stream = C.c_void_p(_arrays.current_stream_handle())
    f = downsample_factor(float(radius), pixel_size, "ambient_occlusion")
    sx, sy = abs(float(psx)), abs(float(psy))
    if buf is None:
        def buf(name, n):
            return torch.empty(int(n), device=out.device, dtype=torch.float32)
    ns, it = int(kw.get("num_samples", 16)), float(kw.get("intensity", 1.0))
    if f <= 1:
        view = _arrays.DevView(None, int(src_ptr), int(src_h), int(src_w), int(src_ld), "torch")
        p = make_params(num_samples=ns, radius=float(radius), intensity=it, pixel_size=pixel_size)
        run_ambient_occlusion(view, [whole_tile(src_h, src_w, sx, sy, core)], p, make_plane(out))
        return
    hs, ws = (src_h + f - 1) // f, (src_w + f - 1) // f
    small = buf("os_small", hs * ws)[: hs * ws].view(hs, ws)
    N.check(lib.fsg_downsample_nan_aware(C.c_void_p(src_ptr), int(src_ld), int(src_h), int(src_w), int(f),
                                         C.c_void_p(small.data_ptr()), ws, stream))
    rsmall = buf("os_resp", hs * ws)[: hs * ws].view(hs, ws)
    sview = _arrays.DevView(small, small.data_ptr(), hs, ws, ws, "torch")
    p = make_params(num_samples=ns, radius=max(1.0, float(radius) / float(f)), intensity=it,
                    pixel_size=float(pixel_size) * f)
    run_ambient_occlusion(sview, [whole_tile(hs, ws, sx * f, sy * f)], p, make_plane(rsmall))
    N.check(lib.fsg_upsample_to_shape(C.c_void_p(rsmall.data_ptr()), ws, hs, ws, int(src_h), int(src_w),
                                      int(core[0]), int(core[1]), int(core[2]), int(core[3]),
                                      C.c_void_p(out.data_ptr()), int(out.stride(0)), stream))


def _ray_spatial_into(product, *args, **kwargs):
    fn = _openness_spatial_into if product == "openness" else _ao_spatial_into
    return fn(*args, **kwargs)


def spatial_block(block, product: str, radius, *, pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None, **kw):
    """The spatial block function of ``product`` (smoothing, then the product; openness:
    compute_openness_spatial_block with ``radius`` as the maximum distance; ambient
    occlusion: compute_ambient_occlusion_spatial_block)."""
    v = _arrays.as_device_f32_2d(block)
    if product in RAY_PRODUCTS:
        out = _arrays.empty(v.h, v.w, device=v.tensor.device)
        psx, psy = S.resolve_scales(pixel_size, pixel_scale_x, pixel_scale_y)
        if v.h * v.w:
            _ray_spatial_into(product, v.ptr, v.ld, v.h, v.w, (0, 0, v.h, v.w), radius, kw, pixel_size, psx, psy,
                              out)
        return _arrays.wrap_result(out, v.origin)
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


def compute_openness_spatial_block(block, *, openness_type="positive", num_directions=16, max_distance=50,
                                   pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None):
    """_impl_openness.py:135-164."""
    return spatial_block(block, "openness", max_distance, pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                         pixel_scale_y=pixel_scale_y, openness_type=openness_type,
                         num_directions=int(num_directions))


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


def _count_matches(weights, n: int) -> bool:
    """_weight_count_matches (_nan_utils.py:132-139)."""
    if weights is None or isinstance(weights, (str, bytes)):
        return False
    try:
        return len(weights) == n
    except TypeError:
        return False


class CombinePlan:
    """How per-radius responses become one: ``op`` (N.COMBINE_*), the float32 weight of
    each response (1 for max / min / sum) and the divisor applied at the store (n for the
    plain mean, else 1); ``stack`` keeps the responses as bands."""

    def __init__(self, op: int, weights: List[float], divisor: float = 1.0, stack: bool = False):
        self.op, self.weights, self.divisor, self.stack = op, weights, float(divisor), stack


def combine_plan(product: str, agg, weights, n: int, *, direct: bool = False) -> CombinePlan:
    """The combination of the spatial branches.

    ``direct``: the local multi-radius hillshade (``_combine_direct``,
    algorithms/tile/dask_bridge.py:28-69): max / min / sum, a float32-normalised
    weighted mean, else the mean as a sum of r * f32(1/n).
    hillshade (_impl_hillshade.py:109-131): 'mean' with float32-normalised weights
    (even for one radius), 'min', 'max', anything else the plain mean.
    slope / curvature / openness (``_combine_multiscale_dask``, _nan_utils.py:182-213):
    one response as it is, 'max' / 'min' / 'sum', 'mean' with weights L1-normalised in
    float64, else the plain mean.  The plain mean is the float32 sum divided by n.
    """
    a = str(agg or "mean").lower()
    ones = [1.0] * n
    if a == "stack":
        return CombinePlan(N.COMBINE_WSUM, ones, stack=True)
    if product != "hillshade" and n == 1:
        return CombinePlan(N.COMBINE_WSUM, ones)
    if a == "max":
        return CombinePlan(N.COMBINE_MAX, ones)
    if a == "min":
        return CombinePlan(N.COMBINE_MIN, ones)
    if a == "sum" and (direct or product != "hillshade"):
        return CombinePlan(N.COMBINE_WSUM, ones)
    if a == "mean":
        if product == "hillshade":
            if isinstance(weights, (list, tuple)) and len(weights) == n:
                w = np.asarray(weights, dtype=np.float32)
                if np.isfinite(w).all() and float(w.sum()) > 0:
                    w = w / w.sum()
                    return CombinePlan(N.COMBINE_WSUM, [float(np.float32(x)) for x in w])
        elif _count_matches(weights, n):
            c = clean_normalized_weights(weights)
            if c is not None:
                return CombinePlan(N.COMBINE_WSUM, [float(np.float32(x)) for x in c])
    if direct:
        return CombinePlan(N.COMBINE_WSUM, [float(np.float32(1.0 / float(n)))] * n)
    return CombinePlan(N.COMBINE_WSUM, ones, divisor=float(n))


def spatial_depth(product: str, radius) -> int:
    """depth_for_scale (_impl_hillshade.py:98, _impl_slope.py:62, _impl_curvature.py:85,
    _impl_openness.py:196)."""
    r = float(radius)
    if product in RAY_PRODUCTS:   # _impl_ambient_occlusion.py:182
        return int(r) + 1
    return max(3, int(r * 2 + 2)) if product == "curvature" else max(2, int(r * 2 + 1))


def spatial_scales(product: str, radii) -> List[float]:
    """The scale handed to the block function per radius; openness takes
    ``float(int(max(2, round(r))))`` as its maximum distance (_impl_openness.py:193)."""
    if product == "openness":
        return [float(int(max(2, round(float(r))))) for r in radii]
    if product == "ambient_occlusion":   # _impl_ambient_occlusion.py:180
        return [float(max(1, int(round(float(r))))) for r in radii]
    return [float(r) for r in radii]


def spatial_is_large(product: str, scale, threshold: int) -> bool:
    """is_large: ``int(round(r)) > thr`` (_impl_hillshade.py:103), ``int(md) > thr`` for
    openness (_impl_openness.py:197)."""
    if product in RAY_PRODUCTS:   # _impl_ambient_occlusion.py:183
        return int(scale) > threshold
    return int(round(float(scale))) > threshold


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
                 scratch: dict, global_offset: Tuple[int, int] = (0, 0), agg="mean", stretch=None,
                 mask_nodata: bool = True) -> None:
    """One tile of the spatial product: window (y0, x0, h, w) and core (y0, x0, h, w) in
    raster coordinates; the combined core is stored into ``plane`` (addressing the core's
    first pixel).  ``global_offset`` is added to raster coordinates to give the global
    pixel coordinates the overview is sampled at.  ``stretch``: openness' (p1, p99 - p1).
    ``mask_nodata``: NaN at the raster's NoData (the tile processor's mask); the
    window-level ``process`` returns the combination unmasked."""
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

    scales = spatial_scales(product, radii)
    plan = combine_plan(product, agg, weights, len(scales))
    if plan.stack:
        raise NotImplementedError("agg='stack' yields one band per radius; the tile loop writes one plane")
    acc = buf("acc", ch * cw)[: ch * cw].view(ch, cw)
    resp = buf("resp", ch * cw)[: ch * cw].view(ch, cw)
    # one reflect padding at the largest depth of the locally computed radii: the padding
    # at a smaller depth d is its centred sub-array (the same reflected samples)
    depths = [max(1, min(spatial_depth(product, r), min(wh, ww) - 1)) for r in scales
              if not (spatial_is_large(product, r, thr) and overview is not None)]
    dmax = max(depths) if depths else 0
    if dmax:
        PH, PW = wh + 2 * dmax, ww + 2 * dmax
        padded = buf("pad", PH * PW)[: PH * PW].view(PH, PW)
        N.check(lib.fsg_pad_reflect(C.c_void_p(raster.ptr), raster.ld, raster.h, raster.w, wy, wx, wh, ww, dmax,
                                    ndv, has_nd, C.c_void_p(padded.data_ptr()), PW, stream))
    for i, (r, w) in enumerate(zip(scales, plan.weights)):
        first = 1 if i == 0 else 0
        direct = plan.op == N.COMBINE_WSUM   # responses of a weighted sum go straight into acc
        if spatial_is_large(product, r, thr) and overview is not None:
            cr = overview.response(product, r, kw, pixel_size, psx, psy)
            tgt, tw_, tf = (acc, w, first) if direct else (resp, 1.0, 1)
            N.check(lib.fsg_sample_coarse_accumulate(
                C.c_void_p(cr.ptr), cr.ld, cr.h, cr.w, C.c_void_p(raster.ptr), raster.ld, raster.h, raster.w,
                cy, cx, ch, cw, cy + int(global_offset[0]), cx + int(global_offset[1]), overview.full[0],
                overview.full[1], ndv, has_nd, C.c_float(tw_), tf, C.c_void_p(tgt.data_ptr()), tgt.stride(0),
                stream))
        else:
            d = max(1, min(spatial_depth(product, r), min(wh, ww) - 1))
            ph, pw = wh + 2 * d, ww + 2 * d
            sub = padded.data_ptr() + 4 * ((dmax - d) * PW + (dmax - d))  # the depth-d padding
            pcore = (d + cy - wy, d + cx - wx, ch, cw)
            if product in RAY_PRODUCTS:
                _ray_spatial_into(product, sub, PW, ph, pw, pcore, r, kw, pixel_size, psx, psy, resp, buf=buf)
            else:
                smooth = buf("smooth", ph * pw)[: ph * pw].view(ph, pw)
                _smooth_into(sub, PW, ph, pw, r, pixel_size, product, smooth)
                _run_product(smooth.data_ptr(), pw, ph, pw, pcore, product, kw, pixel_size, psx, psy, resp)
        if not (direct and spatial_is_large(product, r, thr) and overview is not None):
            N.check(lib.fsg_combine(C.c_void_p(resp.data_ptr()), cw, ch, cw, plan.op, C.c_float(w), first,
                                    C.c_void_p(acc.data_ptr()), cw, stream))
    fin = N.StoreFinish()
    fin.divisor = plan.divisor
    fin.stretch_lo, fin.stretch_scale = 0.0, 0.0
    fin.keep_nodata_values = 0 if mask_nodata else 1
    if product in RAY_PRODUCTS and isinstance(stretch, (tuple, list)) and len(stretch) >= 2 \
            and float(stretch[1]) > 1e-12:
        fin.stretch_lo, fin.stretch_scale = float(stretch[0]), float(stretch[1])
    N.check(lib.fsg_masked_store(C.c_void_p(acc.data_ptr()), cw, C.c_void_p(raster.ptr), raster.ld, raster.h,
                                 raster.w, cy, cx, ch, cw, ndv, has_nd, C.byref(fin), C.byref(plane), stream))


def _stack_tile(v, name, radii, weights, kw, px, psx, psy, overview, origin, stretch):
    """agg='stack': one band per radius, band-first (C, H, W)."""
    torch = _arrays._torch()
    bands = torch.empty((len(radii), v.h, v.w), device=v.tensor.device, dtype=torch.float32)
    scratch: dict = {}
    for k, r in enumerate(radii):
        spatial_tile(v, (0, 0, v.h, v.w), (0, 0, v.h, v.w), name, [r], None, kw, pixel_size=px, psx=psx, psy=psy,
                     nodata=None, overview=overview, plane=S.make_plane(bands[k]), scratch=scratch,
                     global_offset=origin, stretch=stretch, mask_nodata=False)
    return bands


def spatial_stencil(name: str, dem_gpu, params: dict):
    """``process(dem, mode='spatial' | multi-radius)`` of a stencil product or of openness
    on one window.

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
    agg = p.get("agg", "mean")
    stream = C.c_void_p(_arrays.current_stream_handle())
    out = _arrays.empty(v.h, v.w, device=v.tensor.device)
    if v.h * v.w == 0:
        return _arrays.wrap_result(out, v.origin)
    if mode != "spatial":
        # _direct_hillshade local multi-radius branch (_combine_direct)
        radii = p.get("radii") or [1]
        radii = [max(1.0, float(r)) for r in radii]
        resp = [_arrays.as_device_f32_2d(spatial_block(v.tensor, name, r, pixel_size=px, pixel_scale_x=psx,
                                                       pixel_scale_y=psy, **kw)) for r in radii]
        plan = combine_plan("hillshade", agg, p.get("weights"), len(radii), direct=True)
        if plan.stack:
            torch = _arrays._torch()
            return _arrays.wrap_result(torch.stack([x.tensor for x in resp], 0), v.origin)
        if len(radii) == 1:
            return _arrays.wrap_result(resp[0].tensor, v.origin)
        for i, (x, w) in enumerate(zip(resp, plan.weights)):
            N.check(N.lib().fsg_combine(C.c_void_p(x.ptr), x.ld, v.h, v.w, plan.op, C.c_float(w),
                                        1 if i == 0 else 0, C.c_void_p(out.data_ptr()), out.stride(0), stream))
        return _arrays.wrap_result(out, v.origin)
    radii, weights = resolve_spatial_radii_weights(p.get("radii"), p.get("weights"), px)
    if name == "hillshade" and p.get("weights") is not None:
        weights = p.get("weights")   # _impl_hillshade.py:84-87 keeps the caller's weights
    overview = None
    cdem = p.get("_overview_coarse_dem")
    if cdem is not None and p.get("_overview_decimation") is not None and p.get("_tile_origin") is not None:
        overview = _GivenOverview(cdem, float(p["_overview_decimation"]), p.get("_tile_full_shape") or (v.h, v.w))
    origin = p.get("_tile_origin") or (0, 0)
    origin = (int(origin[0]), int(origin[1]))
    stretch = p.get("global_stats") if name in RAY_PRODUCTS else None
    if str(agg or "mean").lower() == "stack":
        return _arrays.wrap_result(_stack_tile(v, name, radii, weights, kw, px, psx, psy, overview, origin, stretch),
                                   v.origin)
    spatial_tile(v, (0, 0, v.h, v.w), (0, 0, v.h, v.w), name, radii, weights, kw, pixel_size=px, psx=psx, psy=psy,
                 nodata=None, overview=overview, plane=S.make_plane(out), scratch={}, global_offset=origin, agg=agg,
                 stretch=stretch, mask_nodata=False)
    return _arrays.wrap_result(out, v.origin)


def spatial_openness(dem_gpu, params: dict):
    """``OpennessAlgorithm.process(dem, mode='spatial')`` on one window (_impl_openness.py:188-216)."""
    return spatial_stencil("openness", dem_gpu, params)


def _product_kwargs(name: str, p: dict) -> dict:
    if name == "hillshade":
        return {"azimuth": float(p.get("azimuth", 315.0)), "altitude": float(p.get("altitude", 45.0)),
                "z_factor": 1.0 if p.get("z_factor") is None else float(p.get("z_factor", 1.0))}
    if name == "slope":
        return {"unit": str(p.get("unit", "degree"))}
    if name == "openness":
        return {"openness_type": str(p.get("openness_type", "positive")),
                "num_directions": int(p.get("num_directions", 16))}
    if name == "ambient_occlusion":
        return {"num_samples": int(p.get("num_samples", 16)), "intensity": float(p.get("intensity", 1.0))}
    return {"curvature_type": str(p.get("curvature_type", "mean"))}


class _GivenOverview(Overview):
    """An overview handed in by the caller (``_overview_coarse_dem``)."""

    def __init__(self, coarse_dem, decimation: float, full_shape):
        self.dem = _arrays.as_device_f32_2d(coarse_dem).tensor
        self.oh, self.ow = int(self.dem.shape[0]), int(self.dem.shape[1])
        self.decimation = float(decimation)
        self.full = (int(full_shape[0]), int(full_shape[1]))
        self._resp = {}
