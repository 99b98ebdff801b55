"""Single-device tile loop: the hot path of ``process_dem_tiles``
(core/tile_processor.py:1027-1745) for an in-memory raster.

The reference runs one ThreadPoolExecutor task per tile (read window ->
NoData->NaN -> H2D -> block function -> crop -> NoData re-mask -> D2H ->
quantise).  Here the whole tile grid is one call per kernel: each tile is an
``fsg_tile`` descriptor (window = core + halo clipped at the raster edge,
per-tile signed pixel scales), outputs land in full-raster planes, NoData
masking and the int16/uint8 encoding run in the kernels' store epilogue.
What stays on the host is the parameter logic the reference runs before the
tile loop: radii/weights resolution, halo sizing, the topousm_fast
large-radius overview split and the global-statistics pre-pass.
File I/O (COG read/write, VRT build) is out of scope: the raster is an array.
"""
from __future__ import annotations

import logging
import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .. import _arrays
from .. import _native as N
from ..algorithms import _impl_ambient_occlusion as AO
from ..algorithms import _impl_openness as OP
from ..algorithms import _impl_topousm_fast as TU
from ..algorithms import _stencil as S
from ..algorithms._stats import robust_unsigned_stretch_stat_func, topousm_fast_stat_func
from ..common.spatial_mode import (LOCAL_RADII, LOCAL_WEIGHTS, auto_spatial_radii, auto_spatial_weights,
                                   deduplicate_radii_weights, normalize_topousm_radii)
from ..io.output_encoding import SUPPORTED_OUTPUT_DTYPES, quantize_params, resolve_output_range
from ..io.raster_info import tile_pixel_scales

logger = logging.getLogger(__name__)

HOT_PATH_ALGORITHMS = ("hillshade", "slope", "curvature", "topousm_fast", "openness", "ambient_occlusion")
SPATIAL_ALGORITHMS = ("hillshade", "slope", "curvature", "openness", "ambient_occlusion")
RAY_ALGORITHMS = ("openness", "ambient_occlusion")
MAX_DEPTH = 150  # algorithms/_base.py:16


@dataclass
class TileInfo:
    """One entry of core/tile_processor.py:1610-1627."""
    ty: int
    tx: int
    core_x: int
    core_y: int
    core_w: int
    core_h: int
    win_x: int
    win_y: int
    win_w: int
    win_h: int


def tile_grid(height: int, width: int, tile_size: int, padding: int) -> List[TileInfo]:
    """Cores of ``tile_size`` with ``padding`` halos clipped (not reflected) at raster edges."""
    out = []
    ny = (height + tile_size - 1) // tile_size
    nx = (width + tile_size - 1) // tile_size
    for ty in range(ny):
        for tx in range(nx):
            cx, cy = tx * tile_size, ty * tile_size
            cw, ch = min(tile_size, width - cx), min(tile_size, height - cy)
            wx, wy = max(cx - padding, 0), max(cy - padding, 0)
            wx1, wy1 = min(cx + cw + padding, width), min(cy + ch + padding, height)
            out.append(TileInfo(ty, tx, cx, cy, cw, ch, wx, wy, wx1 - wx, wy1 - wy))
    return out


def required_padding(algorithm: str, params: dict, sigma: float, tile_size: int) -> int:
    """Halo of core/tile_processor.py:207-383 for the hot-path algorithms."""
    try:
        base = int(math.ceil(max(float(sigma), 0.0) * 5.0))
    except Exception:
        base = 32
    required = max(32, base)
    mode = str(params.get("mode", "spatial")).lower()
    if algorithm == "topousm_fast":
        radii, _ = normalize_topousm_radii(params.get("radii"), params.get("weights"))
        if radii:
            required = max(required, int(max(radii) + 16))
    if mode == "spatial" and algorithm in SPATIAL_ALGORITHMS:
        radii = params.get("radii") or auto_spatial_radii(None)
        radii_f = [float(r) for r in radii if float(r) > 0]
        overview_active = bool(params.get("radii")) and algorithm != "topousm_fast"
        thr = max(256, int(tile_size) // 16)
        if overview_active:
            small = [r for r in radii_f if int(round(r)) <= thr] or [min(radii_f)]
            max_radius = int(round(max(small)))
        else:
            max_radius = max(int(round(r)) for r in radii_f)
        if algorithm in RAY_ALGORITHMS:
            required = max(required, int(max_radius + 16))
        else:
            required = max(required, int(max_radius * 2 + 2))
    return max(32, ((required + 31) // 32) * 32)


def make_tiles(infos: Sequence[TileInfo], *, pixel_scale_x: float, pixel_scale_y: float,
               transform=None, geographic: bool = False) -> List[N.Tile]:
    tiles = []
    for t in infos:
        d = N.Tile()
        d.win_y0, d.win_x0, d.win_h, d.win_w = t.win_y, t.win_x, t.win_h, t.win_w
        d.core_y0, d.core_x0, d.core_h, d.core_w = t.core_y, t.core_x, t.core_h, t.core_w
        d.out_y0, d.out_x0 = t.core_y, t.core_x
        if geographic and transform is not None:
            d.pixel_scale_x, d.pixel_scale_y = tile_pixel_scales(t.core_y, t.core_h, transform)
        else:
            d.pixel_scale_x, d.pixel_scale_y = float(pixel_scale_x), float(pixel_scale_y)
        tiles.append(d)
    return tiles


def _load_algorithm(name: str):
    """core/tile_processor.py:807-820: a new instance of
    ``algorithms/tile/<name>.py``'s class, ``ValueError`` for an unknown name."""
    from ..algorithms.registry import load_algorithm
    return load_algorithm(name)


# --------------------------------------------------------------- global stats
def stratified_windows(width, height, by0, by1, bx0, bx1, *, grid=3, tile=4096):
    """algorithms/_norm_stats.py:64-100: unique grid x grid windows over the valid bbox."""
    cell_h = max(1, (int(by1) - int(by0)) // grid)
    cell_w = max(1, (int(bx1) - int(bx0)) // grid)
    out, seen = [], set()
    for gy in range(grid):
        for gx in range(grid):
            ccy = int(by0) + gy * cell_h + cell_h // 2
            ccx = int(bx0) + gx * cell_w + cell_w // 2
            wy0 = int(min(max(0, ccy - tile // 2), max(0, int(height) - tile)))
            wx0 = int(min(max(0, ccx - tile // 2), max(0, int(width) - tile)))
            tw, th = min(tile, int(width) - wx0), min(tile, int(height) - wy0)
            key = (wy0, wx0, tw, th)
            if key not in seen:
                seen.add(key)
                out.append(key)
    return out


def bbox_sample_indices(H: int, W: int):
    """Rows and columns of the nearest-resampled overview the valid-data box is
    taken from (_norm_stats.py:253-264): index floor((i + 0.5) * n / o), o = n // cov."""
    cov = max(1, max(W, H) // 512)
    oh, ow = max(1, H // cov), max(1, W // cov)
    ys = np.minimum(((np.arange(oh, dtype=np.float64) + 0.5) * (H / oh)).astype(np.int64), H - 1)
    xs = np.minimum(((np.arange(ow, dtype=np.float64) + 0.5) * (W / ow)).astype(np.int64), W - 1)
    return ys, xs, cov


def _valid_bbox(dem_dev, nodata, sample=None) -> Optional[Tuple[int, int, int, int]]:
    """Valid-data bounding box from a nearest-resampled overview (_norm_stats.py:253-264);
    ``sample`` = ((H, W), that overview as a device array) when the raster is not on the device."""
    torch = _arrays._torch()
    if sample is not None:
        (H, W), ov = sample
        cov = bbox_sample_indices(H, W)[2]
    else:
        H, W = dem_dev.shape
        ys, xs, cov = bbox_sample_indices(H, W)
        ov = dem_dev.index_select(0, torch.from_numpy(ys).to(dem_dev.device)).index_select(
            1, torch.from_numpy(xs).to(dem_dev.device))
    valid = torch.isfinite(ov)
    if nodata is not None and not math.isnan(float(nodata)):
        valid &= ~((ov - float(nodata)).abs() <= 1e-6)
    if not bool(valid.any()):
        return None
    yy = torch.nonzero(valid.any(dim=1)).flatten()
    xx = torch.nonzero(valid.any(dim=0)).flatten()
    by0, by1 = int(yy.min()) * cov, min(H, (int(yy.max()) + 1) * cov)
    bx0, bx1 = int(xx.min()) * cov, min(W, (int(xx.max()) + 1) * cov)
    return by0, by1, bx0, bx1


def global_stats_prepass(dem_dev, algorithm: str, params: dict, *, nodata=None, grid: int = 3,
                         max_tile: int = 4096, min_valid_frac: float = 0.02, shard=None, source=None):
    """Full-resolution stratified-window statistics (_norm_stats.py:176-298).

    Runs the algorithm's raw block function on up to grid^2 windows (one GPU
    call over all windows), trims each by its margin, pools the valid values
    and returns the algorithm's stats: topousm_fast -> (p99|x|,), openness and
    ambient occlusion -> (p1, p99 - p1).  Returns None when no window qualifies.
    With a ``shard`` (core.sharding.Shard) each rank evaluates its round-robin
    share of the windows and the statistics of the union come from the exact
    histogram merge: every rank returns the numbers one device would.
    ``source`` (a ``(shape, window_fn, bbox)`` triple) replaces ``dem_dev`` when
    the raster is not on the device: ``window_fn(y0, x0, h, w)`` returns a window
    as a device array, ``bbox`` the valid-data box (or None).
    """
    torch = _arrays._torch()
    if source is not None:
        (H, W), window_fn, bbox_src = source
    else:
        H, W = dem_dev.shape
        window_fn = lambda y0, x0, h, w: dem_dev[y0:y0 + h, x0:x0 + w]  # noqa: E731
    if algorithm == "topousm_fast":
        radii = params.get("_topousm_fast_full_radii") or params.get("radii")
        max_scale = max(float(r) for r in radii)
    else:
        # _norm_stat_max_scale (_norm_stats.py:103-121): the largest of the radii, the
        # radius and the maximum distance the parameters carry
        vals = []
        if isinstance(params.get("radii"), (list, tuple)) and params.get("radii"):
            vals.append(max(float(r) for r in params["radii"]))
        for key in ("radius", "max_distance"):
            if params.get(key):
                vals.append(float(params[key]))
        if algorithm == "openness" and not params.get("max_distance"):
            vals.append(50.0)   # the block function's default distance
        if algorithm == "ambient_occlusion" and not params.get("radius"):
            vals.append(10.0)   # the block function's default radius
        max_scale = max(vals) if vals else 16.0
    margin = max(1, int(max_scale + 16))
    tile = max(min(2048, max_tile), 4 * margin)
    bbox = bbox_src if source is not None else _valid_bbox(dem_dev, nodata)
    if bbox is None:
        return None
    wins = stratified_windows(W, H, *bbox, grid=grid, tile=min(tile, max(W, H)))
    if shard is not None:
        wins = shard.mine(wins)
    pooled = []
    nanmask_needed = nodata is not None and not (isinstance(nodata, float) and math.isnan(nodata))
    for wy0, wx0, tw, th in wins:
        a = window_fn(wy0, wx0, th, tw)
        if nanmask_needed:
            a = torch.where((a - float(nodata)).abs() <= 1e-6, torch.full_like(a, float("nan")), a)
        if float(torch.isfinite(a).float().mean()) < min_valid_frac:
            continue
        if algorithm == "topousm_fast":
            w = params.get("_topousm_fast_full_weights") or params.get("weights")
            raw = TU.compute_topousm_fast_efficient_block(a, radii=radii, weights=w,
                                                          pixel_size=float(params.get("pixel_size", 1.0)))
        elif algorithm == "ambient_occlusion":
            raw, _ = AO.ambient_occlusion_plane(a, num_samples=params.get("num_samples", 16),
                                                radius=params.get("radius", 10.0),
                                                intensity=params.get("intensity", 1.0),
                                                pixel_size=params.get("pixel_size", 1.0),
                                                pixel_scale_x=params.get("pixel_scale_x"),
                                                pixel_scale_y=params.get("pixel_scale_y"))
        else:
            raw, _, _ = OP.openness_planes(a, openness_type=params.get("openness_type", "positive"),
                                           num_directions=params.get("num_directions", 16),
                                           max_distance=params.get("max_distance", 50),
                                           pixel_size=params.get("pixel_size", 1.0),
                                           pixel_scale_x=params.get("pixel_scale_x"),
                                           pixel_scale_y=params.get("pixel_scale_y"))
        m = int(min(margin, raw.shape[0] // 3, raw.shape[1] // 3))
        if m > 0:
            raw = raw[m:-m, m:-m]
        pooled.append(raw.reshape(-1))
    if shard is not None:
        from . import sharding as SH
        vals = torch.cat(pooled) if pooled else torch.empty(0, device="cuda")
        if int(shard.allreduce(np.array([len(pooled)], dtype=np.int64))[0]) == 0:
            return None
        if algorithm == "topousm_fast":
            st = SH.sharded_topousm_stat(SH.DeviceHistograms(vals, absolute=True),
                                         lambda: vals.cpu().numpy(), shard.allreduce)
        else:
            finite = torch.where(torch.isfinite(vals), vals, torch.full_like(vals, float("nan")))
            st = SH.sharded_stretch_stat(SH.DeviceHistograms(finite), shard.allreduce)
    else:
        if not pooled:
            return None
        vals = torch.cat(pooled)
        if algorithm == "topousm_fast":
            st = topousm_fast_stat_func(vals)
        else:
            st = robust_unsigned_stretch_stat_func(vals)
    if not st or not math.isfinite(float(st[-1])) or float(st[-1]) <= 1e-9:
        return None
    return st


# ------------------------------------------------------------------ the loop
@dataclass
class LoopResult:
    output: object                  # float32 plane or integer code plane (device tensor)
    dtype: str
    quantize: Optional[dict]
    tiles: int
    padding: int
    stats: Optional[tuple] = None
    extras: Dict[str, object] = field(default_factory=dict)
    rows: Tuple[int, int] = (0, 0)  # raster rows this process wrote (its band when sharded)


def resolve_run(algorithm: str, H: int, W: int, algo_params: dict, *, output_dtype: str, output_range,
                pixel_size, pixel_scale_x, pixel_scale_y, multiscale_mode: bool):
    """The parameter logic the reference runs before its tile loop: output encoding,
    pixel scales, local / spatial radii and weights (core/tile_processor.py:1027-1281).
    Returns (params, quantise params, output dtype, px, psx, psy, spatial)."""
    params = dict(algo_params)
    qp = None
    if output_dtype in ("int16", "uint8"):
        rng = resolve_output_range(algorithm, params=params, override=output_range)
        if rng is None:
            logger.warning("No fixed output range for %s; writing float32 instead of %s.", algorithm, output_dtype)
            output_dtype = "float32"
        else:
            qp = quantize_params(rng[0], rng[1], output_dtype)
    px = float(pixel_size) if pixel_size else 1.0
    psx = float(pixel_scale_x) if pixel_scale_x is not None else px
    psy = float(pixel_scale_y) if pixel_scale_y is not None else -px
    params["pixel_size"] = px
    mode = str(params.get("mode", "spatial")).lower()
    is_local = mode == "local" or (algorithm == "topousm_fast" and not multiscale_mode)
    if is_local:
        params["radii"], params["weights"] = list(LOCAL_RADII), list(LOCAL_WEIGHTS)
    elif not params.get("radii"):
        r = auto_spatial_radii(min(H, W))
        params["radii"] = r
        if not params.get("weights"):
            params["weights"] = auto_spatial_weights(len(r))
    spatial = mode == "spatial" and algorithm in SPATIAL_ALGORITHMS
    if spatial:
        dr, dw = sanitize_spatial_radii_weights(algorithm, params.get("radii"), params.get("weights"))
        if dr is not None:
            params["radii"] = dr
            if dw is not None:
                params["weights"] = dw
            elif params.get("weights") is not None:
                params["weights"] = None

    return params, qp, output_dtype, px, psx, psy, spatial


def topousm_split(params: dict, H: int, W: int, tile_size: int, overview_fn) -> None:
    """topousm_fast's large-radius overview split (core/tile_processor.py:1236-1281):
    radii above max(256, tile/16) leave the per-tile list and become one coarse
    field on the <= 2048 px overview that ``overview_fn(oh, ow)`` returns."""
    full_r, full_w = normalize_topousm_radii(params.get("radii"), params.get("weights"))
    if full_w is None and full_r:
        full_w = [1.0 / len(full_r)] * len(full_r)
    params["radii"], params["weights"] = full_r, full_w
    thr = TU.topousm_fast_default_large_radius_threshold(int(tile_size))
    sr, sw, lr, lw = TU.split_radii_by_threshold(full_r, full_w, thr)
    if lr:
        scale = max(W / 2048.0, H / 2048.0, 1.0)
        ow, oh = max(1, int(round(W / scale))), max(1, int(round(H / scale)))
        coarse_dem = overview_fn(oh, ow)
        field = TU.compute_topousm_fast_large_coarse_field(coarse_dem, large_radii=lr, large_weights=lw,
                                                           decimation=float(scale))
        params.update({"_topousm_fast_full_radii": list(full_r), "_topousm_fast_full_weights": list(full_w),
                       "radii": sr, "weights": sw, "_topousm_fast_coarse_field": field,
                       "_topousm_fast_small_radii": sr, "_topousm_fast_small_weights": sw,
                       "_topousm_fast_w_large": float(sum(lw)), "_topousm_fast_full_shape": (H, W)})


def process_dem_array(dem, algorithm: str, *, tile_size: int = 4096, padding: Optional[int] = None,
                      sigma: float = 10.0, pixel_size: Optional[float] = None, pixel_scale_x: Optional[float] = None,
                      pixel_scale_y: Optional[float] = None, transform=None, geographic: bool = False,
                      nodata: Optional[float] = None, output_dtype: str = "float32", output_range=None,
                      multiscale_mode: bool = True, shard="auto", **algo_params) -> LoopResult:
    """Run one hot-path algorithm over an in-memory raster with the reference's tile semantics.

    ``dem``: 2-D float32 host (NumPy) or device array.  ``transform``: the
    (a, b, c, d, e, f) affine of a geographic raster (per-tile metric scales).
    Returns full-raster planes on the device.

    ``shard``: ``"auto"`` (default) runs sharded when a torch.distributed process
    group of more than one rank is initialised, a ``core.sharding.Shard`` runs as
    that rank, ``None`` / ``False`` runs the whole raster.  A sharded rank writes
    the cores of its band of tile rows (``LoopResult.rows``; the other rows keep
    the NoData value) and takes the global statistics from the exact cross-rank
    merge, so the union of the bands equals the single-device result.
    """
    if algorithm not in HOT_PATH_ALGORITHMS:
        raise ValueError(f"{algorithm!r} is not on the GB300 hot path ({', '.join(HOT_PATH_ALGORITHMS)})")
    torch = _arrays._torch()
    v = _arrays.as_device_f32_2d(dem, name="dem")
    H, W = v.h, v.w
    output_dtype = str(output_dtype or "float32").lower()
    if output_dtype not in SUPPORTED_OUTPUT_DTYPES:
        raise ValueError(f"Unsupported output_dtype={output_dtype!r}. Choose from {SUPPORTED_OUTPUT_DTYPES}.")
    params, qp, output_dtype, px, psx, psy, spatial = resolve_run(
        algorithm, H, W, algo_params, output_dtype=output_dtype, output_range=output_range, pixel_size=pixel_size,
        pixel_scale_x=pixel_scale_x, pixel_scale_y=pixel_scale_y, multiscale_mode=multiscale_mode)
    if algorithm == "topousm_fast":
        topousm_split(params, H, W, tile_size, lambda oh, ow: TU.overview(v.tensor, (oh, ow), nodata=nodata))

    if shard == "auto":
        from .sharding import shard_from_environment
        shard = shard_from_environment()
    elif shard is False:
        shard = None
    pad = required_padding(algorithm, params, sigma, tile_size) if padding is None else int(padding)
    infos = tile_grid(H, W, int(tile_size), pad)
    if shard is not None:
        from .sharding import shard_tiles
        infos = shard_tiles(infos, shard.world, shard.rank)
    tiles = make_tiles(infos, pixel_scale_x=psx, pixel_scale_y=psy, transform=transform, geographic=geographic)
    out = _arrays.empty(H, W, output_dtype, device=v.tensor.device)
    if shard is not None or spatial:
        # rows of other ranks, and spatial-mode tiles skipped for NoData, keep the NoData
        # value; otherwise the local kernels write every core pixel of the covering grid
        out.fill_(0 if output_dtype != "float32" else float("nan"))
    rows = (min((t.core_y for t in infos), default=0), max((t.core_y + t.core_h for t in infos), default=0))
    res = LoopResult(out, output_dtype, qp, len(tiles), pad, rows=rows)

    if spatial:
        stretch = None
        if algorithm in RAY_ALGORITHMS:
            # the openness / AO stats describe the local display value (max_distance / radius)
            # in every mode (_norm_stats.py:42-46, :195-283)
            stretch = params.get("global_stats")
            if stretch is None:
                stretch = global_stats_prepass(v.tensor, algorithm, dict(params, pixel_scale_x=psx,
                                                                         pixel_scale_y=psy), nodata=nodata,
                                               shard=shard)
            res.stats = stretch
        _spatial_loop(v, infos, tiles, algorithm, params, px, nodata, out, output_dtype, qp, stretch)
    else:
        stats = params.get("global_stats")
        if (stats is None or (algorithm == "topousm_fast" and not stats)) and \
                algorithm in ("topousm_fast", "ambient_occlusion", "openness"):
            stats = global_stats_prepass(v.tensor, algorithm, dict(params, pixel_scale_x=psx, pixel_scale_y=psy),
                                         nodata=nodata, shard=shard)
        if algorithm in ("topousm_fast", "ambient_occlusion", "openness"):
            res.stats = stats
        launch_local(algorithm, v, tiles, params, px, nodata, S.make_plane(out, output_dtype, qp), stats, (H, W))
    return res


def launch_local(algorithm: str, v, tiles, params: dict, px: float, nodata, plane, stats, full_shape) -> None:
    """The kernel call of a local-mode product (and of topousm_fast) over a tile list:
    ``v`` the raster view the tiles address, ``plane`` the output plane in raster
    coordinates, ``stats`` the global statistics (None: raw / unstretched)."""
    if algorithm in ("hillshade", "slope", "curvature"):
        name = {"hillshade": "hillshade", "slope": "slope"}.get(algorithm)
        if algorithm == "curvature":
            ct = params.get("curvature_type", "mean")
            name = "curvature_" + (ct if ct in ("mean", "gaussian", "planform") else "profile")
        sp = S.make_params(azimuth=params.get("azimuth", 315.0), altitude=params.get("altitude", 45.0),
                           z_factor=params.get("z_factor", 1.0), pixel_size=px, nodata=nodata,
                           unit=params.get("unit", "degree"))
        S.launch(v, tiles, sp, {S.OUTPUT_INDEX[name]: plane})
    elif algorithm == "topousm_fast":
        scale = float(stats[0]) if stats else 0.0
        tp, keep = TU.make_params(params["radii"], params["weights"] or [], px, nodata=nodata,
                                  coarse=params.get("_topousm_fast_coarse_field"),
                                  w_large=params.get("_topousm_fast_w_large", 0.0), full_shape=full_shape,
                                  scale=scale, path=params.get("topousm_path", "exact"))
        TU.run_topousm(v, tiles, tp, plane)
    elif algorithm == "ambient_occlusion":
        ap = AO.make_params(num_samples=params.get("num_samples", 16), radius=params.get("radius", 10.0),
                            intensity=params.get("intensity", 1.0), pixel_size=px, nodata=nodata, stretch=stats)
        AO.run_ambient_occlusion(v, tiles, ap, plane)
    else:  # openness
        op = OP.make_params(openness_type=params.get("openness_type", "positive"),
                            num_directions=params.get("num_directions", 16),
                            max_distance=params.get("max_distance", 50), pixel_size=px,
                            sampling=params.get("sampling", "reference"), nodata=nodata, stretch=stats)
        OP.run_openness(v, tiles, op, plane)


def sanitize_spatial_radii_weights(algorithm: str, radii, weights):
    """_sanitize_spatial_radii_weights_for_tile (core/tile_processor.py:102-172).

    Stencil products: integer radii >= 1, duplicates merged with their weights.
    openness and ambient occlusion: integer radii >= 2 (non-positive ones dropped with
    their weights),
    weights kept only when every kept radius has one, then de-duplicated.
    Returns (radii, weights) or (None, weights) when no radius survives.
    """
    if not isinstance(radii, (list, tuple)) or len(radii) == 0:
        return None, weights
    if algorithm not in RAY_ALGORITHMS:
        ints = []
        for r in radii:
            try:
                fv = float(r)
            except (TypeError, ValueError):
                continue
            if fv > 0:
                ints.append(max(1, int(round(fv))))
        if not ints:
            return None, weights
        return deduplicate_radii_weights(ints, weights)
    out_r, out_w = [], []
    for i, rv in enumerate(radii):
        try:
            r = int(round(float(rv)))
        except (TypeError, ValueError):
            continue
        if r <= 0:
            continue
        out_r.append(max(2, r))
        if isinstance(weights, (list, tuple)) and i < len(weights):
            try:
                out_w.append(float(weights[i]))
            except (TypeError, ValueError):
                out_w.append(0.0)
    if not out_r:
        return None, None
    return deduplicate_radii_weights(out_r, out_w if len(out_w) == len(out_r) else None)


def _spatial_loop(v, infos, tiles, algorithm, params, px, nodata, out, output_dtype, qp, stretch=None):
    """Spatial mode of a stencil product or of openness over the tile grid (one
    spatial_tile per tile; large radii from one shared overview)."""
    from ..algorithms import _spatial as SP
    from ..common.spatial_mode import resolve_spatial_radii_weights
    radii, weights = resolve_spatial_radii_weights(params.get("radii"), params.get("weights"), px)
    if algorithm == "hillshade" and params.get("weights") is not None:
        weights = params.get("weights")   # _impl_hillshade.py:84-87 keeps the caller's weights
    kw = SP._product_kwargs(algorithm, params)
    overview = None
    if radii and max(int(round(float(r))) for r in radii) > 256:
        overview = SP.Overview(v, nodata=nodata)
    agg = params.get("agg", "mean")
    scratch: dict = {}
    for info, t in zip(infos, tiles):
        plane = S.make_plane(out[info.core_y:info.core_y + info.core_h, info.core_x:info.core_x + info.core_w],
                             output_dtype, qp)
        SP.spatial_tile(v, (info.win_y, info.win_x, info.win_h, info.win_w),
                        (info.core_y, info.core_x, info.core_h, info.core_w), algorithm, radii, weights, kw,
                        pixel_size=px, psx=float(t.pixel_scale_x), psy=float(t.pixel_scale_y), nodata=nodata,
                        overview=overview, plane=plane, scratch=scratch, agg=agg, stretch=stretch)
