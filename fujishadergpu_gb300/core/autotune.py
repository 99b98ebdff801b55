"""Tile-shape autotuner for the batched tile loop.

The reference picks its tile size from presets and the free memory of the
device (config/auto_tune.py:120-176).  Here the choice is measured: for each
product and raster (overview level) the candidate tile sizes are timed on a
sample window of that raster through the same prepared launches the batch
uses, and the fastest per output pixel wins.  Results are cached in a JSON
file keyed by GPU name, product, parameters and raster shape
(``FSG_AUTOTUNE_CACHE`` overrides the default
``~/.cache/fujishadergpu_gb300/autotune.json``; ``FSG_AUTOTUNE=0`` disables
measuring and takes the first candidate that fits).
"""
from __future__ import annotations

import json
import os
import threading
from typing import Callable, Dict, Optional, Sequence

DEFAULT_CANDIDATES = (256, 512, 1024, 2048, 4096)


def default_cache_path() -> str:
    env = os.environ.get("FSG_AUTOTUNE_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "fujishadergpu_gb300", "autotune.json")


class Autotuner:
    """choose(key, candidates, measure) -> the candidate with the lowest measured cost.

    ``measure(candidate)`` returns a cost (seconds per output pixel, or any
    comparable number; None = candidate not applicable).  Decisions are cached
    in memory and, when ``path`` is set, in a JSON file shared across runs."""

    def __init__(self, path: Optional[str] = None, enabled: Optional[bool] = None):
        self.path = path if path is not None else default_cache_path()
        self.enabled = (os.environ.get("FSG_AUTOTUNE", "1") != "0") if enabled is None else bool(enabled)
        self._lock = threading.Lock()
        self._cache: Dict[str, dict] = {}
        self.measured: Dict[str, Dict[str, float]] = {}
        if self.path and os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    data = json.load(f)
                if isinstance(data, dict):
                    self._cache = {k: v for k, v in data.items() if isinstance(v, dict) and "choice" in v}
            except (OSError, ValueError):
                self._cache = {}

    @staticmethod
    def key(*parts) -> str:
        return "|".join(str(p) for p in parts)

    def choose(self, key: str, candidates: Sequence[int], measure: Callable[[int], Optional[float]]) -> int:
        cands = [int(c) for c in candidates]
        if not cands:
            raise ValueError("no candidate tile sizes")
        with self._lock:
            hit = self._cache.get(key)
        if hit is not None and int(hit["choice"]) in cands:
            return int(hit["choice"])
        if not self.enabled:
            return cands[0]
        costs: Dict[str, float] = {}
        for c in cands:
            v = measure(c)
            if v is not None:
                costs[str(c)] = float(v)
        if not costs:
            return cands[0]
        best = int(min(costs, key=lambda k: costs[k]))
        with self._lock:
            self._cache[key] = {"choice": best, "costs": costs}
            self.measured[key] = costs
            self._save_locked()
        return best

    def _save_locked(self) -> None:
        if not self.path:
            return
        try:
            os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
            tmp = self.path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(self._cache, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except OSError:
            pass  # a read-only cache location only costs re-measuring

    def cached(self, key: str) -> Optional[int]:
        with self._lock:
            hit = self._cache.get(key)
        return int(hit["choice"]) if hit is not None else None


__all__ = ["Autotuner", "DEFAULT_CANDIDATES", "default_cache_path"]
