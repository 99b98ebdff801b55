"""Constants and the algorithm base class (algorithms/_base.py:12-53)."""
from __future__ import annotations

from abc import ABC, abstractmethod


class Constants:
    DEFAULT_GAMMA = 1 / 2.2
    DEFAULT_AZIMUTH = 315
    DEFAULT_ALTITUDE = 45
    MAX_DEPTH = 150


class TileAlgorithm(ABC):
    """Tile-side algorithm interface (algorithms/tile_shared.py:19-44):
    ``process(dem_gpu, **params)`` takes one halo window as a CUDA device
    array and returns the result for the whole window."""

    @abstractmethod
    def process(self, dem_gpu, **params):
        ...

    @abstractmethod
    def get_default_params(self) -> dict:
        ...

    def _merged(self, params: dict) -> dict:
        """algorithms/tile/dask_bridge.py:16-25: defaults overlaid by params."""
        merged = dict(self.get_default_params())
        merged.update(params)
        return merged
