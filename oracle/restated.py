"""CPU oracle: a NumPy/SciPy restatement of FujiShaderGPU's raster hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the ``fujishadergpu_gb300`` package
imports this module; it is used by ``tests/`` (as the checker), by
``__graft_entry__.smoke()`` and by the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` (as the timed CPU implementation of the path).

Every function restates one reference function (cited as
``path:line`` inside the FujiShaderGPU source tree) step by step, keeping the
reference's float32 operation order so that the restatement reproduces the
reference's own outputs (``tests/golden`` holds those outputs, generated from
the reference itself; ``tests/test_oracle_golden.py`` pins this module to
them).  Passing ``dtype=np.float64`` runs the same steps in float64: that is
the FP64 oracle against which the GPU kernels' error is stated.

The reference runs on CuPy; here ``cupy`` is NumPy and ``cupyx.scipy.ndimage``
is ``scipy.ndimage``.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
from scipy import ndimage as ndi

GAMMA = 1.0 / 2.2          # algorithms/_base.py:13
DEFAULT_AZIMUTH = 315      # algorithms/_base.py:14
DEFAULT_ALTITUDE = 45      # algorithms/_base.py:15


# =============================================================================
# NoData, NaN fill and gradients
# =============================================================================
def nodata_mask(data: np.ndarray, nodata: Optional[float]) -> Optional[np.ndarray]:
    """core/tile_processor.py:185-196: NaN, or |v - nodata| <= 1e-6 (rtol 0), or NaN."""
    if nodata is None:
        return None
    if isinstance(nodata, float) and math.isnan(nodata):
        return np.isnan(data)
    return np.isclose(data, float(nodata), rtol=0.0, atol=1e-6) | np.isnan(data)


def _nan_aware_smooth(block, filt, zero_where_no_weight=True):
    """Normalised convolution shared by _nan_utils.py:18-31 and :34-47.

    ``filt`` is the linear filter.  Without NaN the plain filter is returned;
    otherwise filt(values with NaN->0) / filt(valid weights), 0 where the
    weight is 0.
    """
    nan = np.isnan(block)
    if not nan.any():
        return filt(block), nan
    zero = block.dtype.type(0)
    values = np.where(nan, zero, block)
    valid = (~nan).astype(block.dtype)
    num = filt(values * valid)
    den = filt(valid)
    with np.errstate(invalid="ignore", divide="ignore"):
        out = np.where(den > 0, num / den, 0)
    return out.astype(block.dtype, copy=False), nan


def gaussian_mean_nan_aware(block, sigma=1.0, mode="nearest"):
    """_nan_utils.py:18-31 (handle_nan_with_gaussian)."""
    return _nan_aware_smooth(block, lambda a: ndi.gaussian_filter(a, sigma=sigma, mode=mode))


def box_mean_nan_aware(block, size, mode="reflect"):
    """_nan_utils.py:34-47 (handle_nan_with_uniform)."""
    return _nan_aware_smooth(block, lambda a: ndi.uniform_filter(a, size=size, mode=mode))


def _steps(pixel_size, psx, psy, absolute=True):
    """Step sizes of _nan_utils.py:67-72 (absolute) / _impl_curvature.py:263-268 (signed)."""
    sy = float(psy if psy is not None else pixel_size)
    sx = float(psx if psx is not None else pixel_size)
    if absolute:
        sy, sx = abs(sy), abs(sx)
    if abs(sy) < 1e-9:
        sy = float(pixel_size if pixel_size else 1.0)
    if abs(sx) < 1e-9:
        sx = float(pixel_size if pixel_size else 1.0)
    return sy, sx


def nan_aware_gradient(block, *, scale=1.0, pixel_size=1.0, psx=None, psy=None):
    """_nan_utils.py:50-74 (handle_nan_for_gradient).

    NaN cells are filled with the NaN-aware sigma=1 Gaussian mean (only when
    some cell is valid; an all-NaN window becomes zeros), then
    ``np.gradient(filled*scale, |sy|, |sx|, edge_order=2)``.
    """
    nan = np.isnan(block)
    if nan.any():
        if (~nan).any():
            fill, _ = gaussian_mean_nan_aware(block, 1.0, "nearest")
            filled = np.where(nan, fill, block)
        else:
            filled = np.zeros_like(block)
    else:
        filled = block
    sy, sx = _steps(pixel_size, psx, psy, absolute=True)
    dy, dx = np.gradient(filled * scale, sy, sx, edge_order=2)
    return dy, dx, nan


def _restore_nan(out, nan):
    """_nan_utils.py:701-705."""
    if nan.any():
        out[nan] = np.nan
    return out


# =============================================================================
# 3x3-class stencil products
# =============================================================================
def hillshade(block, *, azimuth=DEFAULT_AZIMUTH, altitude=DEFAULT_ALTITUDE, z_factor=1.0,
              pixel_size=1.0, psx=None, psy=None):
    """algorithms/_impl_hillshade.py:20-54 (compute_hillshade_block)."""
    dy, dx, nan = nan_aware_gradient(block, scale=z_factor, pixel_size=pixel_size, psx=psx, psy=psy)
    east = dx * (1.0 if (psx is None or float(psx) >= 0.0) else -1.0)
    north = dy * (1.0 if (psy is None or float(psy) >= 0.0) else -1.0)
    one = block.dtype.type(1.0)
    norm = np.sqrt(east * east + north * north + one)
    alt = np.radians(altitude)
    az = np.radians(float(azimuth))
    lx = np.sin(az) * np.cos(alt)
    ly = np.cos(az) * np.cos(alt)
    lz = np.sin(alt)
    hs = ((-east * lx) + (-north * ly) + lz) / norm
    hs = np.clip(hs, 0.0, 1.0).astype(block.dtype)
    return _restore_nan(hs, nan)


def slope(block, *, unit="degree", pixel_size=1.0, psx=None, psy=None):
    """algorithms/_impl_slope.py:19-35 (compute_slope_block)."""
    dy, dx, nan = nan_aware_gradient(block, scale=1, pixel_size=pixel_size, psx=psx, psy=psy)
    rad = np.arctan(np.sqrt(dx ** 2 + dy ** 2))
    if unit == "degree":
        out = np.degrees(rad)
    elif unit == "percent":
        out = np.tan(rad) * 100
    else:
        out = rad
    out = _restore_nan(out, nan)
    return out.astype(block.dtype)


def curvature(block, *, curvature_type="mean", pixel_size=1.0, psx=None, psy=None, raw=False):
    """algorithms/_impl_curvature.py:19-57 (compute_curvature_block).

    First derivatives use |pixel scale|; the second ``np.gradient`` uses the
    SIGNED scales (``:263-273``), as the reference does.  ``raw=True`` returns
    the curvature before the tanh/gamma display mapping.
    """
    sy, sx = _steps(pixel_size, psx, psy, absolute=False)
    dy, dx, nan = nan_aware_gradient(block, pixel_size=pixel_size, psx=sx, psy=sy)
    dyy, dyx = np.gradient(dy, sy, sx, edge_order=2)
    dxy, dxx = np.gradient(dx, sy, sx, edge_order=2)
    if curvature_type == "mean":
        p, q, r = dx, dy, dxx
        s = (dxy + dyx) / 2
        t = dyy
        den = np.power(1 + p ** 2 + q ** 2, 1.5)
        num = (1 + q ** 2) * r - 2 * p * q * s + (1 + p ** 2) * t
        k = -num / (2 * den + 1e-10)
    elif curvature_type == "gaussian":
        k = (dxx * dyy - dxy ** 2) / np.power(1 + dx ** 2 + dy ** 2, 2)
    elif curvature_type == "planform":
        k = -(dy ** 2 * dxx - 2 * dx * dy * dxy + dx ** 2 * dyy) / (np.power(dx ** 2 + dy ** 2, 1.5) + 1e-10)
    else:
        k = -(dx ** 2 * dxx + 2 * dx * dy * dxy + dy ** 2 * dyy) / (
            (dx ** 2 + dy ** 2) * np.power(1 + dx ** 2 + dy ** 2, 1.5) + 1e-10)
    if raw:
        return _restore_nan(k.astype(block.dtype), nan)
    disp = np.power((np.tanh(k * 100) + 1) / 2, GAMMA)
    return _restore_nan(disp, nan).astype(block.dtype)


# =============================================================================
# Multiscale helpers
# =============================================================================
_ALGO_FACTOR = {  # _nan_utils.py:571-581
    "topousm_fast": 1.15, "hillshade": 1.0, "slope": 1.0, "specular": 1.4,
    "atmospheric_scattering": 1.05, "curvature": 1.1, "ambient_occlusion": 1.5,
    "openness": 1.4, "multi_light_uncertainty": 1.25,
}


def downsample_factor(radius, *, pixel_size=1.0, algorithm="default", base_radius=24.0, max_factor=16):
    """_nan_utils.py:555-601 (_radius_to_downsample_factor)."""
    r = max(1.0, float(radius))
    px = max(1e-3, float(pixel_size) if pixel_size else 1.0)
    score = (r / max(1.0, base_radius)) * float(_ALGO_FACTOR.get(str(algorithm), 1.0)) * 1.0 \
        * (max(1.0, 1.0 / px) ** 0.35)
    if score <= 1.0:
        return 1
    return int(max(1, min(2 ** int(np.floor(np.log2(score))), max_factor)))


def downsample_nan_aware(block, factor):
    """_nan_utils.py:604-668 (_downsample_nan_aware).

    NaN-aware f x f block mean (ragged edge padded with NaN), then enclosed
    coarse voids (Gaussian valid weight > 0.5, sigma = max(1, min(shape)/64),
    mode nearest) filled with the normalised Gaussian; exterior voids stay NaN.
    """
    if factor <= 1:
        return block
    dt = block.dtype.type
    f = int(factor)
    h, w = block.shape
    oh = max(1, (h + f - 1) // f)
    ow = max(1, (w + f - 1) // f)
    work = block
    if oh * f - h or ow * f - w:
        work = np.pad(work, ((0, oh * f - h), (0, ow * f - w)), mode="constant", constant_values=np.nan)
    cells = work.reshape(oh, f, ow, f)
    fin = np.isfinite(cells)
    cnt = fin.sum(axis=(1, 3), dtype=block.dtype)
    tot = np.where(fin, cells, dt(0)).sum(axis=(1, 3), dtype=block.dtype)
    with np.errstate(invalid="ignore", divide="ignore"):
        coarse = np.where(cnt > 0, tot / np.maximum(cnt, dt(1)), dt(np.nan)).astype(block.dtype)
    cnan = np.isnan(coarse)
    if cnan.any():
        sigma = max(1.0, float(min(coarse.shape)) / 64.0)
        sv = ndi.gaussian_filter(np.where(cnan, dt(0), coarse).astype(block.dtype), sigma=sigma, mode="nearest")
        sw = ndi.gaussian_filter((~cnan).astype(block.dtype), sigma=sigma, mode="nearest")
        enclosed = cnan & (sw > dt(0.5))
        smooth = sv / np.maximum(sw, dt(1e-6))
        coarse = np.where(enclosed, smooth, coarse).astype(block.dtype)
    return coarse.astype(block.dtype)


def upsample_to_shape(block, shape):
    """_nan_utils.py:671-698 (_upsample_to_shape): corner-aligned bilinear zoom."""
    th, tw = int(shape[0]), int(shape[1])
    h, w = block.shape
    dt = block.dtype.type
    if h == th and w == tw:
        return block
    zy = th / max(1, h)
    zx = tw / max(1, w)
    nan = np.isnan(block)
    if not nan.any():
        out = ndi.zoom(block, zoom=(zy, zx), order=1, mode="nearest").astype(block.dtype)
    else:
        valid = (~nan).astype(block.dtype)
        filled = np.where(nan, dt(0), block).astype(block.dtype)
        num = ndi.zoom(filled, zoom=(zy, zx), order=1, mode="nearest")
        den = ndi.zoom(valid, zoom=(zy, zx), order=1, mode="nearest")
        with np.errstate(invalid="ignore", divide="ignore"):
            out = np.where(den > dt(1e-3), num / np.maximum(den, dt(1e-6)), dt(np.nan)).astype(block.dtype)
    ph, pw = max(0, th - out.shape[0]), max(0, tw - out.shape[1])
    if ph or pw:
        out = np.pad(out, ((0, ph), (0, pw)), mode="edge")
    return out[:th, :tw]


def smooth_for_radius(block, radius, *, pixel_size=1.0, algorithm="default"):
    """_nan_utils.py:527-552 (_smooth_for_radius), spatial-mode pre-smoothing."""
    r = max(1.0, float(radius))
    if r <= 1.0:
        return block
    f = downsample_factor(r, pixel_size=pixel_size, algorithm=algorithm)
    if f <= 1:
        out, _ = gaussian_mean_nan_aware(block, max(0.5, r / 2.0), "nearest")
        return out
    small = downsample_nan_aware(block, f)
    sm, _ = gaussian_mean_nan_aware(small, max(0.5, (r / f) / 2.0), "nearest")
    return upsample_to_shape(sm, block.shape)


# =============================================================================
# Spatial mode of the stencil products
# =============================================================================
SPATIAL_PRODUCTS = ("hillshade", "slope", "curvature", "openness")


def stencil_product(block, product, *, pixel_size=1.0, psx=None, psy=None, azimuth=DEFAULT_AZIMUTH,
                    altitude=DEFAULT_ALTITUDE, z_factor=1.0, unit="degree", curvature_type="mean"):
    """The local block function of one stencil product."""
    if product == "hillshade":
        return hillshade(block, azimuth=azimuth, altitude=altitude, z_factor=z_factor, pixel_size=pixel_size,
                         psx=psx, psy=psy)
    if product == "slope":
        return slope(block, unit=unit, pixel_size=pixel_size, psx=psx, psy=psy)
    return curvature(block, curvature_type=curvature_type, pixel_size=pixel_size, psx=psx, psy=psy)


def openness_spatial_block(block, *, openness_type="positive", num_directions=16, max_distance=50,
                           pixel_size=1.0, psx=None, psy=None):
    """_impl_openness.py:135-164 (compute_openness_spatial_block): openness of the NaN-aware
    f x f decimated block (f from the radius, algorithm factor 1.4) with the distance divided
    and the pixel scales multiplied by f, zoomed back to the block's shape."""
    f = downsample_factor(float(max_distance), pixel_size=pixel_size, algorithm="openness")
    if f <= 1:
        return openness(block, openness_type=openness_type, num_directions=num_directions,
                        max_distance=max_distance, pixel_size=pixel_size, psx=psx, psy=psy)
    small = downsample_nan_aware(block, f)
    res = openness(small, openness_type=openness_type, num_directions=num_directions,
                   max_distance=max(2, int(round(float(max_distance) / float(f)))),
                   pixel_size=float(pixel_size) * float(f),
                   psx=None if psx is None else abs(float(psx)) * f,
                   psy=None if psy is None else abs(float(psy)) * f)
    return upsample_to_shape(res, block.shape)


def spatial_block(block, product, radius, *, pixel_size=1.0, **kw):
    """compute_hillshade_spatial_block (_impl_hillshade.py:57-67), compute_slope_spatial_block
    (_impl_slope.py:38-45), _curv_spatial (_impl_curvature.py:72-78): smooth, then the product;
    openness: compute_openness_spatial_block with ``radius`` as the maximum distance."""
    if product == "openness":
        return openness_spatial_block(block, max_distance=radius, pixel_size=pixel_size, **kw)
    if product == "ambient_occlusion":
        return ambient_occlusion_spatial_block(block, radius=radius, pixel_size=pixel_size, **kw)
    sm = smooth_for_radius(block, radius, pixel_size=pixel_size, algorithm=product)
    return stencil_product(sm, product, pixel_size=pixel_size, **kw)


def spatial_depth(product, radius):
    """depth_for_scale of the spatial branches (_impl_hillshade.py:98, _impl_slope.py:62,
    _impl_curvature.py:85, _impl_openness.py:196)."""
    r = float(radius)
    if product in ("openness", "ambient_occlusion"):   # _impl_ambient_occlusion.py:182
        return int(r) + 1
    if product == "curvature":
        return max(3, int(r * 2 + 2))
    return max(2, int(r * 2 + 1))


def spatial_scales(product, radii):
    """The per-radius scale handed to the block function: the radius itself, for openness
    ``float(int(max(2, round(r))))`` (_impl_openness.py:193)."""
    if product == "openness":
        return [float(int(max(2, round(float(r))))) for r in radii]
    if product == "ambient_occlusion":   # _impl_ambient_occlusion.py:180
        return [float(max(1, int(round(float(r))))) for r in radii]
    return [float(r) for r in radii]


def spatial_is_large(product, scale, threshold):
    """is_large of the spatial branches: ``int(round(r)) > thr`` (_impl_hillshade.py:103,
    _impl_slope.py:63, _impl_curvature.py:86), ``int(md) > thr`` for openness (:197)."""
    if product in ("openness", "ambient_occlusion"):   # _impl_ambient_occlusion.py:183
        return int(scale) > threshold
    return int(round(float(scale))) > threshold


def map_overlap_reflect(fn, block, depth):
    """dask ``map_overlap(fn, depth, boundary='reflect')`` on a one-chunk array, with the
    depth cap of _nan_utils.py:502-503 (``max(1, min(depth, min_chunk - 1))``).

    dask's 'reflect' boundary mirrors the array including its edge sample (NumPy's
    'symmetric' pad); the block function runs on the padded chunk and the depth is
    trimmed from every side.
    """
    d = max(1, min(int(depth), min(block.shape) - 1))
    out = fn(np.pad(block, d, mode="symmetric"))
    return out[d:-d, d:-d]


def spatial_large_threshold(window_shape):
    """large_radius_threshold (_nan_utils.py:219-228) of a one-chunk window."""
    return int(max(256, int(min(window_shape)) // 16))


def overview_decimation(full_h, full_w, oh, ow):
    """read_overview_coarse_dem's decimation (_nan_utils.py:862-864)."""
    return 0.5 * (full_w / float(ow) + full_h / float(oh))


def overview_shape(full_h, full_w, sample_max=2048):
    """read_overview_coarse_dem's overview size (_nan_utils.py:846-852)."""
    scale = max(full_w / sample_max, full_h / sample_max, 1.0)
    return max(1, int(round(full_h / scale))), max(1, int(round(full_w / scale)))


def coarse_spatial_response(coarse_dem, product, radius, decimation, *, pixel_size=1.0, psx=None, psy=None, **kw):
    """The overview branch of coarse_large_radius_response (_nan_utils.py:366-395): the block
    function once on the whole overview, radius and pixel scales scaled by the decimation."""
    fac = float(decimation)
    rc = max(1, int(round(float(radius) / fac)))
    return spatial_block(coarse_dem, product, rc, pixel_size=float(pixel_size) * fac,
                         psx=None if psx is None else float(psx) * fac,
                         psy=None if psy is None else float(psy) * fac, **kw).astype(np.float32)


def _plain_mean(responses):
    """da.mean(stack, axis=0) of float32 responses: the float32 sum in order, / float32(n)."""
    out = responses[0].astype(np.float32)
    for r in responses[1:]:
        out = out + r
    return (out / np.float32(len(responses))).astype(np.float32)


def combine_responses(responses, weights, product, agg="mean"):
    """The combination of the spatial branches' per-radius responses.

    hillshade (_impl_hillshade.py:109-131): 'mean' with float32 weights normalised in
    float32, 'min', 'max', anything else the plain mean; slope / curvature / openness
    (_combine_multiscale_dask, _nan_utils.py:182-213): one response returned as it is,
    'max' / 'min' / 'sum' over the stack (NaN propagating), 'mean' with weights
    L1-normalised in float64.  A weighted mean is ``out = r0*w0; out = out + ri*wi`` in
    float32; weights of the wrong length or without a positive sum give the plain mean.
    """
    agg = str(agg or "mean").lower()
    if product != "hillshade" and len(responses) == 1:
        return responses[0]
    if agg == "max":
        return np.max(np.stack(responses, 0), axis=0).astype(np.float32)
    if agg == "min":
        return np.min(np.stack(responses, 0), axis=0).astype(np.float32)
    if agg == "sum" and product != "hillshade":
        out = responses[0].astype(np.float32)
        for r in responses[1:]:
            out = out + r
        return out
    if agg != "mean" or weights is None or isinstance(weights, (str, bytes)) or len(weights) != len(responses):
        return _plain_mean(responses)
    if product == "hillshade":
        w = np.asarray(weights, dtype=np.float32)
        if not (np.isfinite(w).all() and float(w.sum()) > 0):
            return _plain_mean(responses)
        w = w / w.sum()
        ws = [np.float32(float(x)) for x in w]
    else:
        c = clean_normalized_weights(weights)
        if c is None:
            return _plain_mean(responses)
        ws = [np.float32(x) for x in c]
    out = responses[0] * ws[0]
    for r, w in zip(responses[1:], ws[1:]):
        out = out + r * w
    return out.astype(np.float32)


def direct_multiscale(block, product, radii, weights, **kw):
    """_direct_hillshade's local multi-radius branch (tile/dask_bridge.py:72-108 with
    _combine_direct :28-69): per radius the spatial block, float32-normalised weights."""
    rr = [max(1.0, float(r)) for r in radii]
    resp = [spatial_block(block, product, r, **kw) for r in rr]
    if len(resp) == 1:
        return resp[0]
    return combine_responses(resp, weights, "hillshade")


def spatial_window(window, product, radii, weights, *, origin=(0, 0), full_shape=None, coarse_dem=None,
                   decimation=None, pixel_size=1.0, psx=None, psy=None, return_responses=False, agg="mean",
                   stretch=None, **kw):
    """One tile window of a spatial-mode stencil product on the tile backend
    (dask_bridge.py:334-346 falls back to the product's Dask ``process`` on the window as one
    chunk; multiscale_response_fields, _nan_utils.py:441-524).

    Radii above the window's large-radius threshold come from the overview (``coarse_dem``):
    the product of the whole overview sampled at the window's global pixel centres, NaN at
    the window's NaN; the others are ``map_overlap(spatial_block, depth, 'reflect')``.
    """
    h, w = window.shape
    thr = spatial_large_threshold(window.shape)
    H, W = full_shape if full_shape is not None else window.shape
    out = []
    for r in spatial_scales(product, radii):
        if spatial_is_large(product, r, thr) and coarse_dem is not None:
            cr = coarse_spatial_response(coarse_dem, product, r, decimation, pixel_size=pixel_size,
                                         psx=psx, psy=psy, **kw)
            up = bilinear_sample_coarse(cr, origin[0], origin[0] + h, origin[1], origin[1] + w, H, W)
            out.append(np.where(np.isnan(window), np.float32(np.nan), up).astype(np.float32))
        else:
            fn = (lambda b, rr=float(r): spatial_block(b, product, rr, pixel_size=pixel_size, psx=psx, psy=psy,
                                                       **kw))
            out.append(map_overlap_reflect(fn, window, spatial_depth(product, r)).astype(np.float32))
    comb = combine_responses(out, weights, product, agg)
    if product in ("openness", "ambient_occlusion"):
        # apply_display_stretch_dask after the combination (_impl_openness.py:216,
        # _impl_ambient_occlusion.py:203)
        comb = apply_stretch(comb, stretch)
    return (comb, out) if return_responses else comb


# =============================================================================
# topousm_fast
# =============================================================================
def local_mean_for_radius(block, radius, *, pixel_size=1.0):
    """The per-radius local mean of _impl_topousm_fast.py:68-87."""
    f = downsample_factor(float(radius), pixel_size=pixel_size, algorithm="topousm_fast")
    if f > 1:
        small = downsample_nan_aware(block, f)
        rs = max(1, int(round(float(radius) / f)))
        if rs <= 1:
            m, _ = gaussian_mean_nan_aware(small, 1.0, "nearest")
        else:
            m, _ = box_mean_nan_aware(small, 2 * rs + 1, "reflect")
        return upsample_to_shape(m, block.shape)
    if radius <= 1:
        m, _ = gaussian_mean_nan_aware(block, 1.0, "nearest")
        return m
    m, _ = box_mean_nan_aware(block, 2 * radius + 1, "reflect")
    return m


def topousm_block(block, *, radii, weights=None, pixel_size=1.0):
    """_impl_topousm_fast.py:49-100 (compute_topousm_fast_efficient_block)."""
    nan = np.isnan(block)
    if weights is None:
        weights = [1.0 / len(radii)] * len(radii)
    if len(weights) != len(radii):
        raise ValueError(f"Length of weights ({len(weights)}) must match length of radii ({len(radii)})")
    w = np.asarray(weights, dtype=block.dtype)
    acc = None
    for radius, wi in zip(radii, w):
        diff = wi * (block - local_mean_for_radius(block, radius, pixel_size=pixel_size))
        acc = diff if acc is None else acc + diff
    return _restore_nan(acc, nan)


def split_radii_by_threshold(radii, weights, threshold):
    """_impl_topousm_fast.py:113-130."""
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


def large_radius_threshold(tile_size):
    """_impl_topousm_fast.py:103-110 / core/tile_processor.py threshold max(256, tile//16)."""
    return int(max(256, int(tile_size) // 16))


def coarse_field(coarse_dem, *, large_radii, large_weights, decimation):
    """_impl_topousm_fast.py:133-155 (compute_topousm_fast_large_coarse_field)."""
    field = None
    dt = coarse_dem.dtype.type
    for r, w in zip(large_radii, large_weights):
        rc = max(1, int(round(float(r) / max(decimation, 1.0))))
        if rc <= 1:
            m, _ = gaussian_mean_nan_aware(coarse_dem, 1.0, "nearest")
        else:
            m, _ = box_mean_nan_aware(coarse_dem, 2 * rc + 1, "reflect")
        term = dt(w) * m
        field = term if field is None else field + term
    return field.astype(coarse_dem.dtype)


def bilinear_sample_coarse(coarse, r0, r1, c0, c1, full_h, full_w, dtype=np.float32):
    """_nan_utils.py:255-281: sample ``coarse`` at global pixel centres, order 1, nearest."""
    ch, cw = coarse.shape
    f = np.dtype(dtype).type
    rr = (np.arange(r0, r1, dtype=dtype) + f(0.5)) * f(ch / float(full_h)) - f(0.5)
    cc = (np.arange(c0, c1, dtype=dtype) + f(0.5)) * f(cw / float(full_w)) - f(0.5)
    coords = np.empty((2, r1 - r0, c1 - c0), dtype=dtype)
    coords[0] = rr[:, None]
    coords[1] = cc[None, :]
    return ndi.map_coordinates(coarse, coords, order=1, mode="nearest").astype(dtype)


def topousm_tile(block, *, radii, weights, pixel_size, coarse=None, small_radii=None,
                 small_weights=None, w_large=0.0, offset=(0, 0), full_shape=None):
    """algorithms/tile/dask_bridge.py:225-259 (_direct_topousm_fast) before normalisation."""
    if coarse is None:
        return topousm_block(block, radii=radii, weights=weights, pixel_size=pixel_size)
    dt = block.dtype.type
    h, w = block.shape
    fh, fw = full_shape if full_shape is not None else block.shape
    large = dt(w_large) * block - bilinear_sample_coarse(
        coarse, offset[0], offset[0] + h, offset[1], offset[1] + w, fh, fw, dtype=block.dtype)
    if small_radii:
        return topousm_block(block, radii=small_radii, weights=small_weights, pixel_size=pixel_size) + large
    return large.astype(block.dtype)


def topousm_scale(data):
    """_normalization.py:21-32 (topousm_fast_stat_func): p99(|x|) of valid values."""
    v = data[~np.isnan(data)]
    if len(v) > 0:
        s = float(np.percentile(np.abs(v), 99.0))
        if s > 1e-9:
            return (s,)
        sd = float(np.std(v))
        return (sd if sd > 1e-9 else 1.0,)
    return (1.0,)


def topousm_normalize(block, stats):
    """_global_stats.py:123-153 with _normalization.py:35-41: block / p99, NaN kept."""
    nan = np.isnan(block)
    s = stats[0]
    out = block / s if s > 0 else np.zeros_like(block)
    return _restore_nan(out, nan).astype(np.float32)


# =============================================================================
# openness
# =============================================================================
def openness_distances(max_distance):
    """_impl_openness.py:67-68: unique(int(linspace(0.1, 1, 10) * D)) > 0."""
    d = np.unique((np.linspace(0.1, 1.0, 10) * max_distance).astype(int))
    return d[d > 0]


def openness_offsets(num_directions, max_distance):
    """_impl_openness.py:58-59 and :95-100: (dx, dy) ray offsets, Python round (half-even)."""
    ang = np.linspace(0, 2 * np.pi, num_directions, endpoint=False)
    dirs = np.stack([np.cos(ang), np.sin(ang)], axis=1)
    out = []
    for d in range(num_directions):
        ray = []
        for r in openness_distances(max_distance):
            ox = int(round(float(r) * float(dirs[d][0])))
            oy = int(round(float(r) * float(dirs[d][1])))
            if ox == 0 and oy == 0:
                continue
            ray.append((ox, oy))
        out.append(ray)
    return out


def openness(block, *, openness_type="positive", num_directions=16, max_distance=50,
             pixel_size=1.0, psx=None, psy=None, raw_degrees=False, offsets=None, rows=None):
    """_impl_openness.py:31-132 (compute_openness_vectorized).

    ``raw_degrees=True`` returns the directional mean angle in degrees before the
    /(pi/2), clip and gamma display mapping (the quantity the 0.01 degree
    parity gate is stated on).  ``offsets`` (per direction, a list of (dx, dy))
    replaces the reference's 10 sampled distances, e.g. with every step of the
    ray for the dense ray-march.  ``rows=(y0, y1)`` returns only those output
    rows (the samples still come from the whole block), the same values as
    rows y0..y1 of the full result.
    """
    full = block
    y0, y1 = (0, block.shape[0]) if rows is None else (int(rows[0]), int(rows[1]))
    block = full[y0:y1]
    h, w = block.shape
    nan = np.isnan(block)
    positive = openness_type == "positive"
    init = -np.pi / 2 if positive else np.pi / 2
    sx = abs(float(psx)) if psx is not None else float(pixel_size)
    sy = abs(float(psy)) if psy is not None else float(pixel_size)
    if sx < 1e-9:
        sx = float(pixel_size) if pixel_size else 1.0
    if sy < 1e-9:
        sy = float(pixel_size) if pixel_size else 1.0
    if offsets is None:
        offsets = openness_offsets(num_directions, max_distance)
    D = max([max(abs(ox), abs(oy)) for ray in offsets for ox, oy in ray] or [0])
    zero = block.dtype.type(0)
    if D > 0:
        fnan = np.isnan(full)
        pad = np.pad(np.where(fnan, 0.0, full), D, mode="edge")
        pad_valid = np.pad(~fnan, D, mode="constant", constant_values=False)
    angle_sum = np.zeros((h, w), dtype=block.dtype)
    count = np.zeros((h, w), dtype=block.dtype)
    for ray in offsets:
        ext = np.full((h, w), init, dtype=block.dtype)
        any_valid = np.zeros((h, w), dtype=bool)
        for ox, oy in ray:
            shifted = pad[D + y0 + oy:D + y0 + oy + h, D + ox:D + ox + w]
            sv = pad_valid[D + y0 + oy:D + y0 + oy + h, D + ox:D + ox + w]
            dist = max(float(np.hypot(float(ox) * sx, float(oy) * sy)), 1e-9)
            ang = np.arctan((shifted - block) / dist)
            valid = sv & ~nan
            if positive:
                ext = np.where(valid, np.maximum(ext, ang), ext)
            else:
                ext = np.where(valid, np.minimum(ext, ang), ext)
            any_valid |= valid
        dir_angle = (np.pi / 2 - ext) if positive else (np.pi / 2 + ext)
        angle_sum += np.where(any_valid, dir_angle, 0.0)
        count += any_valid.astype(block.dtype)
    mean = angle_sum / np.maximum(count, 1.0)
    if raw_degrees:
        return _restore_nan(np.degrees(mean).astype(block.dtype), nan)
    op = np.clip(mean / (np.pi / 2), 0, 1)
    out = np.power(op, GAMMA)
    return _restore_nan(out, nan).astype(block.dtype)


def dense_offsets(num_directions, max_distance):
    """Every integer step k = 1..D of each ray (same rounding as the reference's offsets)."""
    ang = np.linspace(0, 2 * np.pi, num_directions, endpoint=False)
    out = []
    for a in ang:
        c, s = float(np.cos(a)), float(np.sin(a))
        ray = []
        for k in range(1, int(max_distance) + 1):
            ox, oy = int(round(k * c)), int(round(k * s))
            if ox == 0 and oy == 0:
                continue
            ray.append((ox, oy))
        out.append(ray)
    return out


def ao_offsets(num_samples, radius):
    """_impl_ambient_occlusion.py:54-88: per ring r = radius * (0.25, 0.5, 0.75, 1.0), the
    offsets (np.round(r cos), np.round(r sin)) of each sample direction (half-even), with the
    ring's distance factor 1 - 0.3 * ring; (0, 0) offsets are skipped."""
    ang = np.linspace(0, 2 * np.pi, num_samples, endpoint=False)
    dirs = np.stack([np.cos(ang), np.sin(ang)], axis=1)
    out = []
    for rf in (0.25, 0.5, 0.75, 1.0):
        r = radius * rf
        dxs = np.round(r * dirs[:, 0]).astype(int)
        dys = np.round(r * dirs[:, 1]).astype(int)
        for i in range(num_samples):
            dx, dy = int(dxs[i]), int(dys[i])
            if dx == 0 and dy == 0:
                continue
            out.append((dx, dy, 1.0 - rf * 0.3))
    return out


def ambient_occlusion(block, *, num_samples=16, radius=10.0, intensity=1.0, pixel_size=1.0,
                      psx=None, psy=None):
    """_impl_ambient_occlusion.py:32-121 (compute_ambient_occlusion_block).

    Edge-padded samples (the block's border values stand in beyond it), elevation angle
    atan(dz / d) clamped to [0, pi/4] and normalised, weighted by the ring's distance
    factor and averaged over the valid samples; AO = clip(1 - mean * intensity, 0, 1),
    NaN cells set to 1, Gaussian sigma 1 ('nearest'), gamma 1/2.2, NaN restored.
    """
    h, w = block.shape
    dt = block.dtype.type
    nan = np.isnan(block)
    sx = abs(float(psx)) if psx is not None else float(pixel_size)
    sy = abs(float(psy)) if psy is not None else float(pixel_size)
    if sx < 1e-9:
        sx = float(pixel_size) if pixel_size else 1.0
    if sy < 1e-9:
        sy = float(pixel_size) if pixel_size else 1.0
    D = max(1, int(round(float(radius))))
    pad = np.pad(block, D, mode="edge")
    total = np.zeros((h, w), dtype=block.dtype)
    count = np.zeros((h, w), dtype=block.dtype)
    for dx, dy, df in ao_offsets(num_samples, radius):
        shifted = pad[D + dy:D + dy + h, D + dx:D + dx + w]
        dist = max(float(np.hypot(float(dx) * sx, float(dy) * sy)), 1e-9)
        ang = np.arctan((shifted - block) / dist)
        occ = np.minimum(np.maximum(0, ang) / (np.pi / 4), 1.0)
        valid = ~(np.isnan(shifted) | nan)
        total += np.where(valid, occ * df, 0)
        count += np.where(valid, 1.0, 0)
    count = np.maximum(count, 1.0)
    mean = total / count
    ao = np.clip(1.0 - mean * intensity, 0, 1)
    if nan.any():
        ao = ndi.gaussian_filter(np.where(nan, 1.0, ao), sigma=1.0, mode="nearest")
    else:
        ao = ndi.gaussian_filter(ao, sigma=1.0, mode="nearest")
    out = np.power(ao, GAMMA)
    return _restore_nan(out, nan).astype(block.dtype)


def ambient_occlusion_spatial_block(block, *, num_samples=16, radius=10.0, intensity=1.0, pixel_size=1.0,
                                    psx=None, psy=None):
    """_impl_ambient_occlusion.py:124-157 (compute_ambient_occlusion_spatial_block): AO of the
    NaN-aware f x f decimated block (f from the radius, algorithm factor 1.5) with the radius
    divided (at least 1) and the pixel scales multiplied by f, zoomed back to the block."""
    f = downsample_factor(float(radius), pixel_size=pixel_size, algorithm="ambient_occlusion")
    if f <= 1:
        return ambient_occlusion(block, num_samples=num_samples, radius=radius, intensity=intensity,
                                 pixel_size=pixel_size, psx=psx, psy=psy)
    small = downsample_nan_aware(block, f)
    res = ambient_occlusion(small, num_samples=num_samples, radius=max(1.0, float(radius) / float(f)),
                            intensity=intensity, pixel_size=float(pixel_size) * float(f),
                            psx=None if psx is None else float(abs(float(psx)) * f),
                            psy=None if psy is None else float(abs(float(psy)) * f))
    return upsample_to_shape(res, block.shape)


def stretch_stats(values):
    """_global_stats.py:181-203 (robust_unsigned_stretch_stat_func): (p1, p99-p1)."""
    if values is None:
        return (0.0, 0.0)
    v = values[np.isfinite(values)]
    if v.size == 0:
        return (0.0, 0.0)
    lo = float(np.percentile(v, 1.0))
    hi = float(np.percentile(v, 99.0))
    sc = hi - lo
    if not (sc > 1e-12):
        return (lo, 0.0)
    return (lo, sc)


def apply_stretch(result, stats):
    """algorithms/tile/dask_bridge.py:173-187 (_apply_display_stretch_block)."""
    if not (isinstance(stats, (tuple, list)) and len(stats) >= 2):
        return result
    lo, sc = float(stats[0]), float(stats[1])
    if not (sc > 1e-12):
        return result
    return np.maximum((result - np.float32(lo)) / np.float32(sc), np.float32(0.0)).astype(np.float32)


# =============================================================================
# Output encoding
# =============================================================================
NORM_HEADROOM = 1.176  # io/output_encoding.py:39
OUTPUT_VALUE_RANGES = {  # io/output_encoding.py:40-73 (hot-path subset)
    "topousm_fast": (-NORM_HEADROOM, NORM_HEADROOM),
    "hillshade": (0.0, 1.0),
    "curvature": (0.0, 1.0),
    "openness": (0.0, 1.0),
    "ambient_occlusion": (0.0, 1.0),
    "slope": (0.0, 90.0),
}
_INT_MAXPOS = {"int16": 32767, "uint8": 255}


def resolve_output_range(algorithm, *, params=None, override=None):
    """io/output_encoding.py:89-127 (hot-path algorithms)."""
    if override is not None:
        lo, hi = float(override[0]), float(override[1])
        if hi > lo:
            return lo, hi
        raise ValueError(f"output range must satisfy high > low, got ({lo!r}, {hi!r})")
    algo = str(algorithm).lower()
    if algo == "slope" and params is not None:
        unit = str(params.get("unit", "degree")).lower()
        if unit == "radian":
            return (0.0, float(np.pi / 2.0))
        if unit != "degree":
            return None
    return OUTPUT_VALUE_RANGES.get(algo)


def quantize_params(lo, hi, dtype):
    """io/output_encoding.py:130-175."""
    lo, hi = float(lo), float(hi)
    dt = str(dtype).lower()
    maxpos = _INT_MAXPOS[dt]
    signed = lo < 0.0 < hi
    if signed:
        a = max(abs(lo), abs(hi))
        a = a if a > 0 else 1.0
        if dt == "int16":
            ac, bc, dmin, dmax = maxpos / a, 0.0, -maxpos, maxpos
        else:
            ac, bc, dmin, dmax = (maxpos - 1) / 2.0 / a, (maxpos + 1) / 2.0, 1, maxpos
    else:
        span = (hi - lo) if (hi - lo) > 0 else 1.0
        ac = (maxpos - 1) / span
        bc = 1.0 - ac * lo
        dmin, dmax = 1, maxpos
    return {"a_coef": float(ac), "b_coef": float(bc), "dn_min": int(dmin), "dn_max": int(dmax),
            "scale": float(1.0 / ac), "offset": float(-bc / ac), "nodata": 0.0, "signed": bool(signed)}


def quantize_array(arr, qp, dtype):
    """io/output_encoding.py:178-190: clip(rint(f32(a)*v + f32(b))), non-finite -> 0."""
    a = np.asarray(arr, dtype=np.float32)
    dn = np.rint(np.float32(qp["a_coef"]) * a + np.float32(qp["b_coef"]))
    dn = np.clip(dn, qp["dn_min"], qp["dn_max"])
    dn = np.where(np.isfinite(a), dn, 0.0)
    return dn.astype(np.dtype(dtype))


# =============================================================================
# Tile geometry, geographic scales, radii / weights
# =============================================================================
def tile_grid(height, width, tile_size, padding):
    """core/tile_processor.py:1610-1627: (ty, tx, core_x, core_y, core_w, core_h,
    win_x, win_y, win_w, win_h); windows are clipped (not reflected) at raster edges."""
    ny = (height + tile_size - 1) // tile_size
    nx = (width + tile_size - 1) // tile_size
    out = []
    for ty in range(ny):
        for tx in range(nx):
            cx, cy = tx * tile_size, ty * tile_size
            cw, ch = min(tile_size, width - cx), min(tile_size, height - cy)
            wx, wy = max(cx - padding, 0), max(cy - padding, 0)
            wx1, wy1 = min(cx + cw + padding, width), min(cy + ch + padding, height)
            out.append((ty, tx, cx, cy, cw, ch, wx, wy, wx1 - wx, wy1 - wy))
    return out


def meters_per_degree(lat_deg):
    """io/raster_info.py:13-35: WGS84 series (m/deg lon, m/deg lat)."""
    lat = math.radians(float(lat_deg))
    m_lat = 111132.92 - 559.82 * math.cos(2.0 * lat) + 1.175 * math.cos(4.0 * lat) - 0.0023 * math.cos(6.0 * lat)
    m_lon = 111412.84 * math.cos(lat) - 93.5 * math.cos(3.0 * lat) + 0.118 * math.cos(5.0 * lat)
    return max(1e-6, float(m_lon)), float(m_lat)


def tile_pixel_scales(core_y, core_h, transform_a, transform_e, y0):
    """core/tile_processor.py:910-932: signed metres per pixel at the core's centre latitude."""
    top = y0 + core_y * transform_e
    bottom = y0 + (core_y + core_h) * transform_e
    lat = 0.5 * (top + bottom)
    mlon, mlat = meters_per_degree(lat)
    px = math.copysign(abs(transform_a) * mlon, transform_a if transform_a != 0 else 1.0)
    py = math.copysign(abs(transform_e) * mlat, transform_e if transform_e != 0 else -1.0)
    return float(px), float(py)


AUTO_RADII_SEQUENCE = (2, 8, 32, 128, 512, 2048)  # algorithms/common/spatial_mode.py:21


def auto_spatial_radii(short_side_px):
    """algorithms/common/spatial_mode.py:60-75."""
    limit = 2048.0 if short_side_px is None else min(2048.0, float(short_side_px) / 10.0)
    r = [x for x in AUTO_RADII_SEQUENCE if float(x) <= limit]
    return list(r) if r else [AUTO_RADII_SEQUENCE[0]]


def auto_spatial_weights(n):
    """algorithms/common/spatial_mode.py:78-84."""
    if n <= 0:
        return []
    raw = [2.0 ** (n - 1 - i) for i in range(n)]
    t = sum(raw)
    return [x / t for x in raw]


def dedup_radii_weights(radii, weights):
    """core/tile_compute.py:9-39 (deduplicate_radii_weights)."""
    order: List[int] = []
    pos: Dict[int, int] = {}
    rl = list(radii)
    for r in rl:
        if r not in pos:
            pos[r] = len(order)
            order.append(r)
    if weights is None:
        return order, None
    wl = list(weights)
    if len(wl) != len(rl):
        return order, None
    agg = [0.0] * len(order)
    for r, v in zip(rl, wl):
        try:
            x = float(v)
        except (TypeError, ValueError):
            x = 0.0
        if not math.isfinite(x) or x <= 0:
            x = 0.0
        agg[pos[r]] += x
    t = sum(agg)
    if t <= 0:
        return order, None
    return order, [x / t for x in agg]


def normalize_topousm_radii(manual_radii, manual_weights, pixel_size):
    """core/tile_compute.py:42-90 with manual radii (the CLI's --radii/--weights)."""
    if manual_radii is None:
        return None, None
    out = []
    for v in manual_radii:
        try:
            x = float(v)
        except (TypeError, ValueError):
            continue
        if not math.isfinite(x):
            continue
        out.append(max(1, int(round(x))))
    if not out:
        return None, None
    return dedup_radii_weights(out, manual_weights)


def clean_normalized_weights(weights):
    """_nan_utils.py:142-154."""
    c = []
    for w in weights:
        try:
            x = float(w)
        except (TypeError, ValueError):
            return None
        c.append(x if np.isfinite(x) and x > 0 else 0.0)
    s = float(sum(c))
    if s <= 0:
        return None
    return [x / s for x in c]


def resolve_spatial_radii_weights(radii, weights, pixel_size, short_side_px=None):
    """_nan_utils.py:77-129 (_normalize_spatial_radii + _resolve_spatial_radii_weights)."""
    def count_ok(ws, n):
        if ws is None or isinstance(ws, (str, bytes)):
            return False
        try:
            return len(ws) == n
        except TypeError:
            return False

    if radii is None:
        ar = auto_spatial_radii(short_side_px)
        aw = auto_spatial_weights(len(ar))
        if count_ok(weights, len(ar)):
            u = clean_normalized_weights(weights)
            if u is not None:
                return ar, u
        return ar, aw
    res = []
    for r in radii:
        try:
            rv = int(round(float(r)))
        except (TypeError, ValueError):
            continue
        if rv > 0:
            res.append(rv)
    if not res:
        res = auto_spatial_radii(None)
    seen = set()
    ordered = []
    for v in res:
        if v not in seen:
            seen.add(v)
            ordered.append(v)
    if count_ok(weights, len(ordered)):
        u = clean_normalized_weights(weights)
        if u is not None:
            return ordered, u
    return ordered, auto_spatial_weights(len(ordered))


__all__ = [n for n in dir() if not n.startswith("_")]


# =============================================================================
# prepare: NoData detection and void fill (io/dem_preprocess.py,
# algorithms/_pyramid_fill.py, utils/nodata_handler.py)
# =============================================================================
FILL_MODES = ("none", "enclosed", "all")   # io/dem_preprocess.py:57

NODATA_SENTINELS = (   # io/dem_preprocess.py:228-238
    0.0, -9999.0, -99999.0, 9999.0,
    -32768.0, 32767.0, -32767.0, 65535.0,
    -2147483648.0, 2147483647.0, -2147483647.0,
    -128.0, 127.0, 255.0,
)


def pushpull_fill(coarse, valid):
    """_pyramid_fill.py:24-84 (pushpull_fill) with NumPy and scipy's zoom: push (x2
    valid-weighted coarsening by zoom order 1 'nearest' until every cell has support or
    the grid is 1x1), pull (zoom back up level by level, filling unsupported cells),
    known cells kept exactly."""
    f32 = np.float32
    out = coarse.astype(f32, copy=True)
    if bool(valid.all()):
        return out
    if not bool(valid.any()):
        return np.zeros_like(out, dtype=f32)
    eps = f32(1e-6)
    w = valid.astype(f32)
    vw = np.where(valid, out, f32(0.0)).astype(f32)
    vws, ws = [vw], [w]
    while max(vws[-1].shape[:2]) > 1 and float(ws[-1].min()) <= 1e-6:
        ch, cw = vws[-1].shape[:2]
        nh, nw = max(1, ch // 2), max(1, cw // 2)
        zy, zx = nh / float(ch), nw / float(cw)
        num = ndi.zoom(vws[-1], zoom=(zy, zx), order=1, mode="nearest")
        den = ndi.zoom(ws[-1], zoom=(zy, zx), order=1, mode="nearest")
        wv = np.minimum(den, f32(1.0))
        mean = np.where(den > eps, num / np.maximum(den, eps), f32(0.0))
        vws.append((mean * wv).astype(f32))
        ws.append(wv.astype(f32))
    filled = np.where(ws[-1] > eps, vws[-1] / np.maximum(ws[-1], eps), f32(0.0)).astype(f32)
    for lvl in range(len(vws) - 2, -1, -1):
        th, tw = vws[lvl].shape[:2]
        fh, fw = filled.shape[:2]
        up = ndi.zoom(filled, zoom=(th / float(fh), tw / float(fw)), order=1, mode="nearest")
        ph, pw = max(0, th - up.shape[0]), max(0, tw - up.shape[1])
        if ph or pw:
            up = np.pad(up, ((0, ph), (0, pw)), mode="edge")
        up = up[:th, :tw]
        wl = ws[lvl]
        vl = np.where(wl > eps, vws[lvl] / np.maximum(wl, eps), f32(0.0))
        filled = np.where(wl > eps, vl, up).astype(f32)
    return np.where(valid, out, filled).astype(f32)


def coarse_shape(width, height, coarse_max):
    """io/dem_preprocess.py:278-282 (_coarse_shape) -> (ch, cw)."""
    scale = max(width / coarse_max, height / coarse_max, 1.0)
    return max(1, int(round(height / scale))), max(1, int(round(width / scale)))


def coarse_oversample(ch, cw, k=4, max_intermediate=4096):
    """io/dem_preprocess.py:537-539 and :156-158: the oversampling of the nearest read."""
    k = max(2, int(k))
    while k > 2 and max(ch * k, cw * k) > int(max_intermediate):
        k -= 1
    return k


def nan_aware_coarse_average(sample, masked, ch, cw, src_nodata, extra_nodata):
    """io/dem_preprocess.py:135-188 (_nan_aware_coarse_average) on an oversampled nearest
    sample (``masked``: the read's own NoData mask) -> (coarse, void mask)."""
    ih, iw = sample.shape
    k = ih // ch
    a = sample.astype(np.float32, copy=False)
    m = masked | ~np.isfinite(a)
    if src_nodata is not None and np.isfinite(src_nodata):
        m = m | (a == np.float32(src_nodata))
    for v in extra_nodata:
        if np.isfinite(v):
            m = m | (a == np.float32(v))
    a = np.where(m, np.nan, a).reshape(ch, k, cw, k)
    finite = np.isfinite(a)
    cnt = finite.sum(axis=(1, 3))
    s = np.nansum(a, axis=(1, 3))
    cmask = cnt == 0
    coarse = np.where(cmask, np.float32(0.0), s / np.maximum(cnt, 1)).astype(np.float32)
    return coarse, cmask


def detect_border_nodata(sample, valid, *, min_border_fraction=0.5, min_total_fraction=0.02):
    """io/dem_preprocess.py:191-225 (_detect_border_nodata)."""
    h, w = sample.shape
    if h < 8 or w < 8:
        return None
    ring = np.concatenate([sample[0, :], sample[-1, :], sample[1:-1, 0], sample[1:-1, -1]])
    ring_valid = np.concatenate([valid[0, :], valid[-1, :], valid[1:-1, 0], valid[1:-1, -1]])
    ring = ring[ring_valid & np.isfinite(ring)]
    if ring.size == 0:
        return None
    vals, counts = np.unique(ring, return_counts=True)
    i = int(np.argmax(counts))
    cand = float(vals[i])
    if counts[i] / ring.size < float(min_border_fraction):
        return None
    if float(np.mean(sample == np.float32(cand))) < float(min_total_fraction):
        return None
    return cand


def detect_sentinel_nodata(sample, valid, *, min_fraction=0.05):
    """io/dem_preprocess.py:241-275 (_detect_sentinel_nodata)."""
    finite = sample[valid & np.isfinite(sample)]
    if finite.size < 64:
        return None
    vals, counts = np.unique(finite, return_counts=True)
    i = int(np.argmax(counts))
    cand = float(vals[i])
    if counts[i] / float(finite.size) < float(min_fraction):
        return None
    known = any(abs(cand - s) <= 1e-6 * max(1.0, abs(s)) for s in NODATA_SENTINELS)
    if known or abs(cand) >= 1e30 or cand == float(vals[0]) or cand == float(vals[-1]):
        return cand
    return None


def edge_connected_mask(mask):
    """utils/nodata_handler.py:13-25 (_edge_connected_mask): masked cells 4-connected to the
    array's border."""
    if not np.any(mask):
        return np.zeros_like(mask, dtype=bool)
    seeds = np.zeros_like(mask, dtype=bool)
    seeds[0, :] = mask[0, :]
    seeds[-1, :] = mask[-1, :]
    seeds[:, 0] = mask[:, 0]
    seeds[:, -1] = mask[:, -1]
    if not np.any(seeds):
        return np.zeros_like(mask, dtype=bool)
    return ndi.binary_propagation(seeds, mask=mask).astype(bool, copy=False)


def sample_coarse_band(surface, exterior, row_off, band_h, width, height, ch, cw):
    """io/dem_preprocess.py:729-767 (_sample_coarse): bilinear samples of the coarse surface
    (and of the exterior mask, > 0.5) at the band's pixel centres, float32 coordinates."""
    rr = (row_off + np.arange(band_h, dtype=np.float32) + np.float32(0.5)) * np.float32(ch / height) \
        - np.float32(0.5)
    cc = (np.arange(width, dtype=np.float32) + np.float32(0.5)) * np.float32(cw / width) - np.float32(0.5)
    coords = np.empty((2, band_h, width), dtype=np.float32)
    coords[0] = rr[:, None]
    coords[1] = cc[None, :]
    fill_vals = ndi.map_coordinates(surface, coords, order=1, mode="nearest", output=np.float32)
    if exterior is None:
        ext = np.zeros((band_h, width), dtype=bool)
    else:
        ext = ndi.map_coordinates(exterior.astype(np.float32), coords, order=1, mode="nearest") > 0.5
    return fill_vals, ext


def apply_band_fill(band, masked, *, row_off, width, height, ch, cw, do_fill, surface, exterior, extra_nodata,
                    fill_mode, out_nodata):
    """io/dem_preprocess.py:770-826 (_apply_band_fill) on one full-width row band
    (``masked``: the read's own NoData mask)."""
    arr = np.array(band, dtype=np.float32, copy=True)
    wmask = masked | ~np.isfinite(arr)
    for v in extra_nodata:
        wmask = wmask | (arr == np.float32(v))
    if wmask.any():
        arr[wmask] = np.float32(np.nan)
    if do_fill and wmask.any():
        fill_vals, ext = sample_coarse_band(surface, exterior, row_off, arr.shape[0], width, height, ch, cw)
        fill_here = wmask & ~ext if fill_mode == "enclosed" else wmask
        arr[fill_here] = fill_vals[fill_here]
    if out_nodata is None:
        if not np.isfinite(arr).all():
            raise RuntimeError(f"fill_mode='all' left {int(np.count_nonzero(~np.isfinite(arr)))} non-finite pixels")
    else:
        arr[~np.isfinite(arr)] = np.float32(np.nan)
    return arr


def nearest_sample(dem, oh, ow):
    """A nearest-neighbour read of ``dem`` at oh x ow: source index floor((i + 0.5) * n / o).
    Stands in for GDAL's NEAREST overview read (absent here; parity of this step unpinned)."""
    h, w = dem.shape
    ys = np.minimum(((np.arange(oh) + 0.5) * (h / oh)).astype(np.int64), h - 1)
    xs = np.minimum(((np.arange(ow) + 0.5) * (w / ow)).astype(np.int64), w - 1)
    # C order, as a raster read returns it: NumPy's float32 reduction order over the
    # coarse cells (and so the rounding of their sums) follows the memory layout
    return np.ascontiguousarray(dem[ys][:, xs])


def prepare_dem(dem, *, nodata=None, fill_mode="enclosed", coarse_max=2048, nodata_override=None,
                detect_nodata=True, nodata_border_fraction=0.5, nodata_sentinel_fraction=0.05):
    """preprocess_dem_to_cog (io/dem_preprocess.py:462-726) on an in-memory raster, minus the
    GDAL/COG I/O: NoData detection on the nearest coarse sample, the NaN-aware coarse
    average, push-pull fill, the exterior mask ('enclosed'), then the full-resolution
    normalise-and-fill of every row (one band: the fill samples global coordinates, so
    bands give the same pixels).  Returns (array, info)."""
    height, width = dem.shape
    ch, cw = coarse_shape(width, height, coarse_max)
    extra = []
    if nodata_override is not None and np.isfinite(nodata_override):
        extra.append(float(nodata_override))
    k = coarse_oversample(ch, cw)
    nn = nearest_sample(dem, ch * k, cw * k).astype(np.float32)
    declared = np.zeros(nn.shape, bool)
    if nodata is not None:
        declared = np.isnan(nn) if np.isnan(nodata) else (nn == np.float32(nodata))
    if detect_nodata:
        nn_valid = (~declared) & np.isfinite(nn)
        for det in (detect_sentinel_nodata(nn, nn_valid, min_fraction=nodata_sentinel_fraction),
                    detect_border_nodata(nn, nn_valid, min_border_fraction=nodata_border_fraction)):
            if det is None:
                continue
            already = any(np.isclose(det, v) for v in extra)
            decl = nodata is not None and np.isclose(det, float(nodata))
            if not already and not decl:
                extra.append(float(det))
    coarse, cmask = nan_aware_coarse_average(nn, declared, ch, cw, nodata, extra)
    cvalid = (~cmask) & np.isfinite(coarse)
    do_fill = fill_mode != "none" and bool((~cvalid).any())
    surface = exterior = None
    if do_fill:
        surface = pushpull_fill(coarse, cvalid)
        if fill_mode == "enclosed":
            exterior = edge_connected_mask(~cvalid)
    out_nodata = None if fill_mode == "all" else float("nan")
    masked = np.zeros(dem.shape, bool)
    if nodata is not None and not np.isnan(nodata):
        masked = dem == np.float32(nodata)
    out = apply_band_fill(dem, masked, row_off=0, width=width, height=height, ch=ch, cw=cw, do_fill=do_fill,
                          surface=surface, exterior=exterior, extra_nodata=extra, fill_mode=fill_mode,
                          out_nodata=out_nodata)
    return out, {"extra_nodata": extra, "coarse_shape": (ch, cw), "oversample": k, "do_fill": do_fill}
