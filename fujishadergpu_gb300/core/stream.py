"""The tile loop over a raster that is read and written in windows
(``process_dem_tiles``, core/tile_processor.py:1027-1745, with its tile
reader / writer, core/tile_io.py:49-72).

The raster stays with a ``TileReader`` (io/tile_io.py); the loop reads one band
of tile rows at a time (the union of the band's windows: cores plus clipped
halos), runs the same kernels as ``process_dem_array`` on the band's tiles and
hands the band's cores to a ``TileWriter``.  The global parameters come from
the reader the way the reference takes them from its file: the statistics
pre-pass reads its stratified windows (algorithms/_norm_stats.py:176-298) and
topousm_fast's large-radius field reads the averaged overview
(algorithms/_nan_utils.py:836-871).  The result equals ``process_dem_array``
on the whole raster (the overview up to its float rounding: the reader
averages in float64 where the device overview kernel uses float-float sums).

Only the local-mode products and topousm_fast stream; spatial mode keeps
whole windows of several radii and runs through ``process_dem_array``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np

from .. import _arrays
from ..algorithms import _stencil as S
from . import tile_loop as TL


@dataclass
class StreamResult:
    tiles: int
    padding: int
    bands: int
    dtype: str
    quantize: Optional[dict]
    stats: Optional[tuple] = None
    rows: Tuple[int, int] = (0, 0)


def _device(a: np.ndarray):
    torch = _arrays._torch()
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32))
    return t.pin_memory().cuda(non_blocking=True)


def process_raster_tiles(reader, writer, algorithm: str, *, tile_size: int = 4096, padding: Optional[int] = None,
                         sigma: float = 10.0, pixel_size: Optional[float] = None, pixel_scale_x: Optional[float] = None,
                         pixel_scale_y: Optional[float] = None, geographic: bool = False,
                         output_dtype: str = "float32", output_range=None, multiscale_mode: bool = True,
                         band_tiles: int = 1, shard="auto", **algo_params) -> StreamResult:
    """Run one hot-path algorithm from ``reader`` to ``writer`` with the reference's tile
    semantics, ``band_tiles`` rows of tiles resident on the device at a time.

    The reader's NoData value and affine transform play the roles of the source file's
    (core/tile_processor.py:185-196, :910-932).  ``shard`` as in ``process_dem_array``:
    a sharded rank streams its band of tile rows only.
    """
    if algorithm not in TL.HOT_PATH_ALGORITHMS:
        raise ValueError(f"{algorithm!r} is not on the GB300 hot path ({', '.join(TL.HOT_PATH_ALGORITHMS)})")
    _arrays.require_cuda()
    torch = _arrays._torch()
    H, W = (int(v) for v in reader.shape)
    nodata = reader.nodata
    if nodata is not None and isinstance(nodata, float) and math.isnan(nodata):
        nodata = None
    output_dtype = str(output_dtype or "float32").lower()
    if output_dtype not in TL.SUPPORTED_OUTPUT_DTYPES:
        raise ValueError(f"Unsupported output_dtype={output_dtype!r}. Choose from {TL.SUPPORTED_OUTPUT_DTYPES}.")
    params, qp, output_dtype, px, psx, psy, spatial = TL.resolve_run(
        algorithm, H, W, algo_params, output_dtype=output_dtype, output_range=output_range, pixel_size=pixel_size,
        pixel_scale_x=pixel_scale_x, pixel_scale_y=pixel_scale_y, multiscale_mode=multiscale_mode)
    if spatial:
        raise ValueError("the streaming tile loop runs local mode and topousm_fast; spatial mode keeps windows "
                         "of several radii: run it through core.tile_loop.process_dem_array")
    if algorithm == "topousm_fast":
        TL.topousm_split(params, H, W, tile_size, lambda oh, ow: _device(reader.read_overview(oh, ow)))
    if shard == "auto":
        from .sharding import shard_from_environment
        shard = shard_from_environment()
    elif shard is False:
        shard = None
    stats = None
    if algorithm in ("topousm_fast", "ambient_occlusion", "openness"):
        stats = params.get("global_stats")
        if stats is None or (algorithm == "topousm_fast" and not stats):
            ys, xs, _ = TL.bbox_sample_indices(H, W)
            bbox = TL._valid_bbox(None, nodata, sample=((H, W), _device(reader.read_rows_cols(ys, xs))))
            source = ((H, W), lambda y0, x0, h, w: _device(reader.read_window(y0, x0, h, w)), bbox)
            stats = TL.global_stats_prepass(None, algorithm, dict(params, pixel_scale_x=psx, pixel_scale_y=psy),
                                            nodata=nodata, shard=shard, source=source)
    pad = TL.required_padding(algorithm, params, sigma, tile_size) if padding is None else int(padding)
    infos = TL.tile_grid(H, W, int(tile_size), pad)
    if shard is not None:
        from .sharding import shard_tiles
        infos = shard_tiles(infos, shard.world, shard.rank)
    rows_of = {}
    for t in infos:
        rows_of.setdefault(t.ty, []).append(t)
    tys = sorted(rows_of)
    esz = {"float32": 4, "int16": 2, "uint8": 1}[output_dtype]
    fill = 0 if output_dtype != "float32" else float("nan")
    nb = 0
    for b in range(0, len(tys), max(1, int(band_tiles))):
        band = [t for ty in tys[b:b + max(1, int(band_tiles))] for t in rows_of[ty]]
        wy0 = min(t.win_y for t in band)
        wy1 = max(t.win_y + t.win_h for t in band)
        cy0 = min(t.core_y for t in band)
        cy1 = max(t.core_y + t.core_h for t in band)
        dev = _device(reader.read_window(wy0, 0, wy1 - wy0, W))
        # The band as rows wy0..wy1-1 of a virtual H x W raster: the tiles keep their raster
        # coordinates (window clipping, geographic scales, the field's global sampling) and
        # the kernels only read inside their windows.
        view = _arrays.DevView(dev, int(dev.data_ptr()) - 4 * wy0 * W, H, W, W, "torch")
        out = _arrays.empty(cy1 - cy0, W, output_dtype, device=dev.device)
        out.fill_(fill)
        plane = S.make_plane(out, output_dtype, qp)
        plane.ptr = int(out.data_ptr()) - esz * cy0 * W
        tiles = TL.make_tiles(band, pixel_scale_x=psx, pixel_scale_y=psy, transform=reader.transform,
                              geographic=geographic)
        TL.launch_local(algorithm, view, tiles, params, px, nodata, plane, stats, (H, W))
        writer.write_window(cy0, 0, out.cpu().numpy())
        del dev, out
        nb += 1
    torch.cuda.synchronize()
    rows = (min((t.core_y for t in infos), default=0), max((t.core_y + t.core_h for t in infos), default=0))
    return StreamResult(len(infos), pad, nb, output_dtype, qp, stats, rows)


__all__ = ["process_raster_tiles", "StreamResult"]
