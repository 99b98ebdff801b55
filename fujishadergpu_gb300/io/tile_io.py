"""Raster tile I/O behind an interface: where the tile loop reads its windows
and writes its cores when the raster is not an in-memory array.

The reference reads each tile window from a COG through rasterio
(``read_tile_window``, core/tile_io.py:49-51), writes each tile's core to its
own GeoTIFF (``write_tile_output``, :54-72) and reads a GDAL average-resampled
overview for its statistics and large-radius field
(algorithms/_nan_utils.py:836-871).  GDAL and rasterio are absent on both
machines this project runs on, so the formats here are:

* ``ArrayReader`` / ``ArrayWriter``: a raster held in host memory;
* ``RawReader`` / ``RawWriter``: a headerless row-major binary raster on disk
  (read through ``numpy.memmap``) with a JSON sidecar for its shape, dtype,
  NoData value and affine transform.

Anything with ``shape``, ``nodata``, ``transform``, ``read_window`` and
``read_overview`` is a reader; anything with ``write_window`` and ``close`` is
a writer (a rasterio-backed pair would implement the same five methods).
``core.stream.process_raster_tiles`` runs the tile loop over such a pair.
"""
from __future__ import annotations

import json
import math
from typing import Optional, Protocol, Sequence, Tuple

import numpy as np


class TileReader(Protocol):
    shape: Tuple[int, int]              # (height, width)
    nodata: Optional[float]
    transform: Optional[Sequence[float]]  # (a, b, c, d, e, f) affine, or None

    def read_window(self, y0: int, x0: int, h: int, w: int) -> np.ndarray:
        """float32 window [y0, y0 + h) x [x0, x0 + w) (inside the raster)."""

    def read_rows_cols(self, rows: np.ndarray, cols: np.ndarray) -> np.ndarray:
        """float32 samples at the outer product of ``rows`` and ``cols``."""

    def read_overview(self, oh: int, ow: int) -> np.ndarray:
        """NaN-aware mean of the source pixels of each cell of an oh x ow grid (cell i
        = pixels [floor(i n / o), floor((i + 1) n / o)), NoData excluded), float32; NaN
        where a cell holds no valid pixel."""


class TileWriter(Protocol):
    def write_window(self, y0: int, x0: int, data: np.ndarray) -> None:
        """Store ``data`` at [y0, y0 + h) x [x0, x0 + w)."""

    def close(self) -> None:
        ...


# ------------------------------------------------------------------ helpers
def _cell_bounds(n: int, o: int) -> np.ndarray:
    """Source index ranges of o cells over n pixels: cell i holds pixels
    [floor(i n / o), floor((i + 1) n / o)) (the device overview's partition)."""
    return (np.arange(o + 1, dtype=np.int64) * n) // o


def _overview_from_bands(read_band, H: int, W: int, oh: int, ow: int, nodata) -> np.ndarray:
    """NaN-aware cell means, accumulated in float64 one band of cell rows at a time."""
    rb, cb = _cell_bounds(H, oh), _cell_bounds(W, ow)
    out = np.full((oh, ow), np.nan, dtype=np.float32)
    for cy in range(oh):
        y0, y1 = int(rb[cy]), int(rb[cy + 1])
        if y1 <= y0:
            continue
        band = np.asarray(read_band(y0, y1 - y0), dtype=np.float32)
        valid = ~np.isnan(band)
        if nodata is not None and not (isinstance(nodata, float) and math.isnan(nodata)):
            valid &= ~(np.abs(band - np.float32(nodata)) <= 1e-6)
        v = np.where(valid, band.astype(np.float64), 0.0)
        s = np.add.reduceat(v.sum(axis=0), cb[:-1]) if W else np.zeros(ow)
        c = np.add.reduceat(valid.sum(axis=0), cb[:-1]) if W else np.zeros(ow)
        empty = np.diff(cb) == 0
        s[empty], c[empty] = 0.0, 0
        with np.errstate(invalid="ignore", divide="ignore"):
            out[cy] = np.where(c > 0, s / np.maximum(c, 1), np.nan).astype(np.float32)
    return out


# ------------------------------------------------------------ in memory
class ArrayReader:
    """A raster held in host memory (any 2-D array convertible to float32)."""

    def __init__(self, data: np.ndarray, *, nodata: Optional[float] = None, transform=None):
        a = np.asarray(data)
        if a.ndim != 2:
            raise ValueError(f"raster must be 2-D, got shape {a.shape}")
        self.data = a
        self.shape = (int(a.shape[0]), int(a.shape[1]))
        self.nodata = nodata
        self.transform = tuple(transform) if transform is not None else None

    def read_window(self, y0, x0, h, w):
        _check_window(self.shape, y0, x0, h, w)
        return np.ascontiguousarray(self.data[y0:y0 + h, x0:x0 + w], dtype=np.float32)

    def read_rows_cols(self, rows, cols):
        return np.ascontiguousarray(self.data[np.asarray(rows)][:, np.asarray(cols)], dtype=np.float32)

    def read_overview(self, oh, ow):
        H, W = self.shape
        return _overview_from_bands(lambda y0, h: self.data[y0:y0 + h], H, W, oh, ow, self.nodata)


class ArrayWriter:
    """Collects written windows in a host array of ``shape`` and ``dtype`` (NoData fill:
    NaN for float32, 0 for the integer codes, as io/output_encoding.py:81-86)."""

    def __init__(self, shape: Tuple[int, int], dtype: str = "float32"):
        dt = np.dtype(dtype)
        self.data = np.full(shape, np.nan if dt.kind == "f" else 0, dtype=dt)

    def write_window(self, y0, x0, data):
        d = np.asarray(data)
        _check_window(self.data.shape, y0, x0, d.shape[0], d.shape[1])
        self.data[y0:y0 + d.shape[0], x0:x0 + d.shape[1]] = d

    def close(self):
        return None


# ------------------------------------------------------------ raw files
def _sidecar(path: str) -> str:
    return path + ".json"


class RawReader:
    """A headerless row-major raster file (``<path>``) with its JSON sidecar
    (``<path>.json``: height, width, dtype, nodata, transform)."""

    def __init__(self, path: str):
        with open(_sidecar(path)) as f:
            meta = json.load(f)
        self.shape = (int(meta["height"]), int(meta["width"]))
        self.nodata = meta.get("nodata")
        self.transform = tuple(meta["transform"]) if meta.get("transform") else None
        self.mm = np.memmap(path, dtype=np.dtype(meta.get("dtype", "float32")), mode="r", shape=self.shape)

    def read_window(self, y0, x0, h, w):
        _check_window(self.shape, y0, x0, h, w)
        return np.ascontiguousarray(self.mm[y0:y0 + h, x0:x0 + w], dtype=np.float32)

    def read_rows_cols(self, rows, cols):
        return np.ascontiguousarray(self.mm[np.asarray(rows)][:, np.asarray(cols)], dtype=np.float32)

    def read_overview(self, oh, ow):
        H, W = self.shape
        return _overview_from_bands(lambda y0, h: self.mm[y0:y0 + h], H, W, oh, ow, self.nodata)


class RawWriter:
    """Creates ``<path>`` (filled with the NoData value) and its sidecar; windows are
    written through a memory map."""

    def __init__(self, path: str, shape: Tuple[int, int], dtype: str = "float32", *, nodata=None, transform=None):
        dt = np.dtype(dtype)
        fill = (np.nan if dt.kind == "f" else 0) if nodata is None else nodata
        meta = {"height": int(shape[0]), "width": int(shape[1]), "dtype": dt.name,
                "nodata": None if (isinstance(fill, float) and math.isnan(fill)) else fill,
                "transform": list(transform) if transform is not None else None}
        with open(_sidecar(path), "w") as f:
            json.dump(meta, f)
        self.mm = np.memmap(path, dtype=dt, mode="w+", shape=tuple(shape))
        self.mm[:] = fill
        self.path = path

    def write_window(self, y0, x0, data):
        d = np.asarray(data)
        _check_window(self.mm.shape, y0, x0, d.shape[0], d.shape[1])
        self.mm[y0:y0 + d.shape[0], x0:x0 + d.shape[1]] = d

    def close(self):
        if self.mm is not None:
            self.mm.flush()
            self.mm = None


def write_raw(path: str, data: np.ndarray, *, nodata=None, transform=None) -> None:
    """Store an array as a raw raster file with its sidecar."""
    w = RawWriter(path, data.shape, np.asarray(data).dtype.name, nodata=nodata, transform=transform)
    w.write_window(0, 0, data)
    w.close()


def _check_window(shape, y0, x0, h, w):
    H, W = int(shape[0]), int(shape[1])
    if h < 0 or w < 0 or y0 < 0 or x0 < 0 or y0 + h > H or x0 + w > W:
        raise ValueError(f"window ({y0}, {x0}, {h}, {w}) outside the {H}x{W} raster")


def read_tile_window(reader: TileReader, tile) -> np.ndarray:
    """The window of one tile (core + clipped halo), as the reference's
    read_tile_window (core/tile_io.py:49-51); ``tile`` is a core.tile_loop.TileInfo."""
    return reader.read_window(tile.win_y, tile.win_x, tile.win_h, tile.win_w)


def write_tile_output(writer: TileWriter, tile, result_core: np.ndarray) -> None:
    """One tile's core, as the reference's write_tile_output (core/tile_io.py:54-72)."""
    writer.write_window(tile.core_y, tile.core_x, result_core)


__all__ = ["TileReader", "TileWriter", "ArrayReader", "ArrayWriter", "RawReader", "RawWriter", "write_raw",
           "read_tile_window", "write_tile_output"]
