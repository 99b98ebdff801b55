"""topousm_fast (algorithms/_impl_topousm_fast.py of the reference).

Block functions keep the reference names; the work is done by ``fsg_topousm``
(per-window multiscale box-mean unsharp mask), ``fsg_topousm_coarse_field``
(large radii on the overview grid) and ``fsg_affine`` (normalisation).
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

from .. import _arrays
from .. import _native as N
from ._base import TileAlgorithm
from ._stats import topousm_fast_stat_func


TopoUSMParams = N.TopoUSMParams


def downsample_factor(radius: float, pixel_size: float) -> int:
    """_radius_to_downsample_factor(radius, pixel_size, 'topousm_fast') (_nan_utils.py:555-601)."""
    return int(N.lib().fsg_topousm_downsample_factor(float(radius), float(pixel_size)))


def make_params(radii: Sequence[int], weights: Sequence[float], pixel_size: float, *, nodata=None,
                coarse=None, w_large: float = 0.0, full_shape=None, scale: float = 0.0, path: str = "exact"):
    """``path``: arithmetic of the full-resolution box means, ``"exact"`` (64-bit
    fixed-point sums on the CUDA cores) or ``"tensor"`` (split-BF16 banded products on
    the tensor cores; tiles holding NoData fall back to the exact kernel)."""
    if path not in N.TOPOUSM_PATHS:
        raise ValueError(f"unknown topousm path {path!r}; choose from {sorted(N.TOPOUSM_PATHS)}")
    n = len(radii)
    rr = (C.c_int32 * max(1, n))(*[int(r) for r in radii])
    ww = (C.c_double * max(1, n))(*[float(w) for w in weights])
    p = TopoUSMParams()
    p.radii = C.cast(rr, C.POINTER(C.c_int32))
    p.weights = C.cast(ww, C.POINTER(C.c_double))
    p.nradii = n
    p.pixel_size = float(pixel_size if pixel_size else 1.0)
    p.has_nodata = 0 if nodata is None else 1
    p.nodata = float("nan") if nodata is None else float(nodata)
    keep = [rr, ww]
    if coarse is not None:
        cv = _arrays.as_device_f32_2d(coarse, name="coarse field")
        keep.append(cv)
        p.coarse_dev = cv.ptr
        p.coarse_ld = cv.ld
        p.coarse_h, p.coarse_w = cv.h, cv.w
        p.full_h, p.full_w = int(full_shape[0]), int(full_shape[1])
        p.w_large = float(w_large)
    p.scale = float(scale)
    p.path = N.TOPOUSM_PATHS[path]
    return p, keep


def run_topousm(view: _arrays.DevView, tiles, params, plane, stream=None):
    tarr = (N.Tile * max(1, len(tiles)))(*tiles)
    s = _arrays.current_stream_handle() if stream is None else stream
    N.check(N.lib().fsg_topousm(C.c_void_p(view.ptr), view.ld, view.h, view.w, tarr, len(tiles), C.byref(params),
                                C.byref(plane), C.c_void_p(s)))


def _window_tile(h, w, off=(0, 0)):
    t = N.Tile()
    t.win_y0, t.win_x0, t.win_h, t.win_w = 0, 0, h, w
    t.core_y0, t.core_x0, t.core_h, t.core_w = 0, 0, h, w
    t.out_y0, t.out_x0 = 0, 0
    return t


def _resolve_weights(radii, weights):
    if weights is None:
        return [1.0 / len(radii)] * len(radii)
    weights = [float(w) for w in weights]
    if len(weights) != len(radii):
        raise ValueError(f"Length of weights ({len(weights)}) must match length of radii ({len(radii)})")
    return weights


def _raw_topousm(block, radii, weights, pixel_size, *, coarse=None, w_large=0.0, offset=(0, 0),
                 full_shape=None, scale=0.0, out_dtype="float32", qp=None, path="exact"):
    from ._stencil import make_plane
    v = _arrays.as_device_f32_2d(block)
    out = _arrays.empty(v.h, v.w, out_dtype, device=v.tensor.device)
    if v.h * v.w == 0:
        return out, v
    params, keep = make_params(radii, weights, pixel_size, coarse=coarse, w_large=w_large,
                               full_shape=full_shape, scale=scale, path=path)
    t = _window_tile(v.h, v.w)
    if coarse is not None:
        # Global origin of the window: fsg_topousm takes it from win_y0/win_x0,
        # so present the block as a window at `offset` of a virtual raster.
        return _raw_with_offset(v, params, keep, offset, full_shape, out, out_dtype, qp), v
    run_topousm(v, [t], params, make_plane(out, out_dtype, qp))
    return out, v


def _raw_with_offset(v, params, keep, offset, full_shape, out, out_dtype, qp):
    """Runs one window whose global origin is ``offset``: the raster pointer is
    moved back by the offset so that window (oy, ox) of the virtual raster is
    the block itself; only the window is ever read."""
    from ._stencil import make_plane
    oy, ox = int(offset[0]), int(offset[1])
    # A virtual raster of (oy + h) x (ox + w) with the block at (oy, ox) and
    # row pitch v.ld: base pointer = block - (oy*ld + ox) elements.
    base = v.ptr - 4 * (oy * v.ld + ox)
    t = N.Tile()
    t.win_y0, t.win_x0, t.win_h, t.win_w = oy, ox, v.h, v.w
    t.core_y0, t.core_x0, t.core_h, t.core_w = oy, ox, v.h, v.w
    t.out_y0, t.out_x0 = 0, 0
    tarr = (N.Tile * 1)(t)
    N.check(N.lib().fsg_topousm(C.c_void_p(base), v.ld, oy + v.h, ox + v.w, tarr, 1, C.byref(params),
                                C.byref(make_plane(out, out_dtype, qp)),
                                C.c_void_p(_arrays.current_stream_handle())))
    return out


def compute_topousm_fast_efficient_block(block, *, radii: Optional[List[int]] = None,
                                         weights: Optional[List[float]] = None, pixel_size: float = 1.0,
                                         path: str = "exact"):
    """Raw multiscale unsharp mask sum_i w_i (z - mean_{r_i}(z)) of one window
    (_impl_topousm_fast.py:49-100).  ``path`` (not in the reference): ``"exact"`` or
    ``"tensor"``, the arithmetic of the full-resolution box means (see make_params)."""
    if radii is None:
        radii = [4, 16, 64]
    radii = [int(r) for r in radii]
    weights = _resolve_weights(radii, weights)
    out, v = _raw_topousm(block, radii, weights, pixel_size, path=path)
    return _arrays.wrap_result(out, v.origin)


def split_radii_by_threshold(radii, weights, threshold):
    """_impl_topousm_fast.py:113-130 (weights keep their absolute values)."""
    n = len(radii)
    if weights is None or len(weights) != n:
        weights = [1.0 / n] * n
    sr, sw, lr, lw = [], [], [], []
    for r, w in zip(radii, weights):
        if int(r) > int(threshold):
            lr.append(int(r))
            lw.append(float(w))
        else:
            sr.append(int(r))
            sw.append(float(w))
    return sr, sw, lr, lw


def topousm_fast_default_large_radius_threshold(min_chunk: int) -> int:
    """_impl_topousm_fast.py:103-110."""
    return int(max(256, int(min_chunk) // 16))


def compute_topousm_fast_large_coarse_field(coarse_dem, *, large_radii, large_weights, decimation):
    """sum_i f32(w_i) * mean_{round(r_i/decimation)}(coarse) (_impl_topousm_fast.py:133-155)."""
    v = _arrays.as_device_f32_2d(coarse_dem, name="coarse_dem")
    out = _arrays.empty(v.h, v.w, device=v.tensor.device)
    n = len(large_radii)
    rr = (C.c_int32 * n)(*[int(r) for r in large_radii])
    ww = (C.c_double * n)(*[float(w) for w in large_weights])
    N.check(N.lib().fsg_topousm_coarse_field(C.c_void_p(v.ptr), v.ld, v.h, v.w, rr, ww, n, float(decimation),
                                             C.c_void_p(out.data_ptr()), out.stride(0),
                                             C.c_void_p(_arrays.current_stream_handle())))
    return _arrays.wrap_result(out, v.origin)


def overview(raster, out_shape, *, nodata=None):
    """NaN-aware block-mean overview of a device raster (the coarse DEM of the large-radius split)."""
    v = _arrays.as_device_f32_2d(raster, name="raster")
    oh, ow = int(out_shape[0]), int(out_shape[1])
    out = _arrays.empty(oh, ow, device=v.tensor.device)
    N.check(N.lib().fsg_overview(C.c_void_p(v.ptr), v.ld, v.h, v.w,
                                 float("nan") if nodata is None else float(nodata), 0 if nodata is None else 1,
                                 C.c_void_p(out.data_ptr()), oh, ow, out.stride(0),
                                 C.c_void_p(_arrays.current_stream_handle())))
    return out


def normalize(raw, stats, *, out_dtype="float32", qp=None):
    """apply_global_normalization(raw, topousm_fast_norm_func, stats) (+ encoding)."""
    from ._stencil import make_plane
    v = _arrays.as_device_f32_2d(raw, name="raw")
    out = _arrays.empty(v.h, v.w, out_dtype, device=v.tensor.device)
    scale = float(stats[0])
    if not scale > 0:
        # topousm_fast_norm_func: zeros_like(block) for a non-positive scale, NaN kept
        torch = _arrays._torch()
        z = torch.where(torch.isnan(v.tensor), v.tensor, torch.zeros_like(v.tensor))
        v = _arrays.as_device_f32_2d(z)
        scale = 0.0
    N.check(N.lib().fsg_affine(C.c_void_p(v.ptr), v.ld, v.h, v.w, 0.0, scale, 0,
                               C.byref(make_plane(out, out_dtype, qp)),
                               C.c_void_p(_arrays.current_stream_handle())))
    return out


class TopoUSMFastAlgorithm(TileAlgorithm):
    """Tile adapter: algorithms/tile/topousm_fast.py -> dask_bridge._direct_topousm_fast (:225-271)."""

    def process(self, dem_gpu, **params):
        p = self._merged(params)
        pixel_size = p.get("pixel_size", 1.0)
        radii = p.get("radii", None)
        weights = p.get("weights", None)
        if radii is None:
            radii = self._determine_optimal_radii(pixel_size)
        coarse = p.get("_topousm_fast_coarse_field", None)
        stats = p.get("global_stats", None)
        stats_ok = isinstance(stats, (tuple, list)) and len(stats) >= 1 and float(stats[0]) > 1e-9
        scale = float(stats[0]) if stats_ok else 0.0
        if coarse is not None:
            small_r = [int(r) for r in (p.get("_topousm_fast_small_radii", []) or [])]
            small_w = p.get("_topousm_fast_small_weights", None)
            small_w = _resolve_weights(small_r, small_w) if small_r else []
            w_large = float(p.get("_topousm_fast_w_large", 0.0))
            off = p.get("_topousm_fast_field_offset", (0, 0))
            v0 = _arrays.as_device_f32_2d(dem_gpu)
            full = p.get("_topousm_fast_full_shape", (v0.h, v0.w))
            out, v = _raw_topousm(dem_gpu, small_r, small_w, pixel_size, coarse=coarse, w_large=w_large,
                                  offset=off, full_shape=full, scale=scale)
        else:
            radii = [int(r) for r in radii]
            out, v = _raw_topousm(dem_gpu, radii, _resolve_weights(radii, weights), pixel_size, scale=scale)
        if not stats_ok:
            # dask_bridge.py:261-270: estimate from this tile only, then normalise
            stats = topousm_fast_stat_func(out)
            out = normalize(out, stats)
        return _arrays.wrap_result(out, v.origin)

    def _determine_optimal_radii(self, pixel_size: float) -> List[int]:
        """_impl_topousm_fast.py:335-347."""
        radii = []
        for dist in (5, 20, 80, 320):
            radii.append(max(2, min(int(dist / pixel_size), 256)))
        return sorted(set(radii))

    def get_default_params(self) -> dict:
        return {"mode": "radius", "radii": None, "weights": None, "sigmas": None, "agg": "mean",
                "auto_sigma": False}
