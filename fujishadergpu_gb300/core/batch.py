"""Batched uneven tiles: one raster and its overview levels through several
hot-path products as one CUDA-graph launch per step.

The reference processes a raster tile by tile on a thread pool
(core/tile_processor.py:1610-1683) and builds overview levels afterwards.
Here an overview pyramid (NaN-aware 2^l x 2^l block means, the reference's
average resampling, algorithms/_nan_utils.py:836-871 restated exactly) is
stacked into one atlas allocation, each level is cut into its own tile grid
(windows clipped at the level's edges, per-tile geographic pixel scales from
the level's transform, core/tile_processor.py:910-932), and every product
becomes one prepared launch (a plan) over the tiles of all levels, or one per
level where the product carries per-level state (topousm_fast's coarse field
and normalisation scale).  The plans' launches are captured once into a CUDA
graph and replayed.  Tile sizes per level and product come from the
autotuner (core/autotune.py), measured on a sample window of that level.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

from .. import _arrays
from .. import _native as N
from ..algorithms import _impl_openness as OP
from ..algorithms import _impl_topousm_fast as TU
from ..algorithms import _stencil as S
from ..io.raster_info import meters_per_degree, tile_pixel_scales
from . import plans as PL
from .autotune import DEFAULT_CANDIDATES, Autotuner
from .tile_loop import TileInfo, global_stats_prepass, required_padding, tile_grid

PRODUCTS = ("hillshade", "topousm_fast", "openness")


@dataclass
class Level:
    index: int
    factor: int          # decimation of this level relative to level 0
    row0: int            # first atlas row
    h: int
    w: int
    transform: Tuple[float, float, float, float, float, float]  # (a, b, c, d, e, f), degrees per pixel

    def pixel_size_m(self) -> float:
        """Mean metric pixel size at the level's centre latitude (the topousm_fast decimation rule's input)."""
        a, _, _, _, e, f = self.transform
        lat = f + 0.5 * self.h * e
        mlon, mlat = meters_per_degree(lat)
        return 0.5 * (abs(a) * mlon + abs(e) * mlat)


class Pyramid:
    """Level 0 and its 2^l overviews stacked vertically in one float32 atlas (row pitch = level-0 width)."""

    def __init__(self, dem, transform, *, levels: int = 3, nodata: Optional[float] = None):
        torch = _arrays._torch()
        v = _arrays.as_device_f32_2d(dem, name="dem")
        H, W = v.h, v.w
        self.nodata = nodata
        self.levels: List[Level] = []
        row = 0
        for li in range(int(levels)):
            f = 1 << li
            h, w = max(1, H // f), max(1, W // f)
            if li > 0 and (h < 2 or w < 2):
                break
            a, b, c, d, e, ff = transform
            self.levels.append(Level(li, f, row, h, w, (a * f, b, c, d, e * f, ff)))
            row += h
        self.atlas = torch.empty((row, W), device=v.tensor.device, dtype=torch.float32)
        self.atlas[:H].copy_(v.tensor)
        nd = 0.0 if nodata is None else float(nodata)
        s = _arrays.current_stream_handle()
        for L in self.levels[1:]:
            # exact NaN-aware f x f block means of level 0 (fsg_overview)
            N.check(N.lib().fsg_overview(C.c_void_p(v.ptr), v.ld, H, W, nd, 0 if nodata is None else 1,
                                         C.c_void_p(self.atlas[L.row0].data_ptr()), L.h, L.w, W, C.c_void_p(s)))
        self.view = _arrays.as_device_f32_2d(self.atlas, name="atlas")

    @property
    def pixels(self) -> int:
        return sum(L.h * L.w for L in self.levels)

    def level_view(self, L: Level):
        return self.atlas[L.row0:L.row0 + L.h, :L.w]


def level_tiles(L: Level, tile_size: int, padding: int) -> Tuple[List[TileInfo], List[N.Tile]]:
    """The level's tile grid (windows clipped at the level's edges) in atlas coordinates."""
    infos = tile_grid(L.h, L.w, int(tile_size), int(padding))
    tiles = []
    for t in infos:
        d = N.Tile()
        d.win_y0, d.win_x0, d.win_h, d.win_w = L.row0 + t.win_y, t.win_x, t.win_h, t.win_w
        d.core_y0, d.core_x0, d.core_h, d.core_w = L.row0 + t.core_y, t.core_x, t.core_h, t.core_w
        d.out_y0, d.out_x0 = L.row0 + t.core_y, t.core_x
        d.pixel_scale_x, d.pixel_scale_y = tile_pixel_scales(t.core_y, t.core_h, L.transform)
        tiles.append(d)
    return infos, tiles


@dataclass
class BatchConfig:
    levels: int = 3
    products: Tuple[str, ...] = PRODUCTS
    topousm_radii: Tuple[int, ...] = (2, 8, 32, 128, 512)
    topousm_weights: Optional[Tuple[float, ...]] = None          # default 2^n, normalised
    openness_distance: int = 256
    openness_directions: int = 16
    azimuth: float = 315.0
    altitude: float = 45.0
    tile_sizes: Optional[Dict[str, Sequence[int]]] = None        # product -> per-level tile size (else autotuned)
    candidates: Tuple[int, ...] = DEFAULT_CANDIDATES
    sample: int = 4096                                           # autotune sample window (px)


@dataclass
class BatchResult:
    outputs: Dict[str, object]
    tile_sizes: Dict[str, List[int]]
    tiles: Dict[str, int]
    stats: Dict[str, list] = field(default_factory=dict)


class BatchedTiles:
    """Hillshade, topousm_fast and openness over a raster and its overviews, as prepared plans.

    ``step()`` launches every plan eagerly; ``capture()`` records them into one
    CUDA graph and ``replay()`` runs the whole step as a single graph launch.
    """

    def __init__(self, dem, transform, *, nodata: Optional[float] = None, config: Optional[BatchConfig] = None,
                 tuner: Optional[Autotuner] = None):
        torch = _arrays._torch()
        self.cfg = cfg = config or BatchConfig()
        self.tuner = tuner if tuner is not None else Autotuner()
        self.pyr = Pyramid(dem, transform, levels=cfg.levels, nodata=nodata)
        self.nodata = nodata
        self.outputs: Dict[str, object] = {}
        self.tile_sizes: Dict[str, List[int]] = {}
        self.tile_counts: Dict[str, int] = {}
        self.stats: Dict[str, list] = {}
        self.plans: List[PL.Plan] = []
        self.plan_products: List[str] = []   # product of each plan
        self._graph: Optional[PL.GraphStep] = None
        shape = tuple(self.pyr.atlas.shape)
        for prod in cfg.products:
            if prod not in PRODUCTS:
                raise ValueError(f"unknown product {prod!r} ({', '.join(PRODUCTS)})")
            self.outputs[prod] = torch.full(shape, float("nan"), device=self.pyr.atlas.device, dtype=torch.float32)
        dev = torch.cuda.get_device_name(self.pyr.atlas.device)
        for prod in cfg.products:
            sizes = []
            for L in self.pyr.levels:
                given = (cfg.tile_sizes or {}).get(prod)
                if given is not None:
                    sizes.append(int(given[min(L.index, len(given) - 1)]))
                else:
                    sizes.append(self._tune(prod, L, dev))
            self.tile_sizes[prod] = sizes
            self._build(prod, sizes)

    # ----------------------------------------------------------- products
    def _topousm_weights(self):
        w = self.cfg.topousm_weights
        if w is None:
            n = len(self.cfg.topousm_radii)
            w = [2.0 ** (n - 1 - i) for i in range(n)]
        s = float(sum(w))
        return [float(x) / s for x in w]

    def _padding(self, prod: str, tile: int) -> int:
        if prod == "hillshade":
            return 8
        if prod == "openness":
            return int(self.cfg.openness_distance) + 32
        # the tile loop pads for the radii left after the large-radius split (core/tile_loop.process_dem_array)
        thr = TU.topousm_fast_default_large_radius_threshold(int(tile))
        sr, sw, _, _ = TU.split_radii_by_threshold(list(self.cfg.topousm_radii), self._topousm_weights(), thr)
        return required_padding("topousm_fast", {"mode": "local", "radii": sr or list(self.cfg.topousm_radii),
                                                 "weights": sw or self._topousm_weights()}, 10.0, tile)

    def _level_plans(self, prod: str, L: Level, tiles: List[N.Tile], out, view, stats=None,
                     level_raster=None) -> List[PL.Plan]:
        """Plans of one product over ``tiles`` (coordinates of ``view``) of level L (or of all levels);
        topousm_fast reads ``level_raster`` (level L as its own raster, rows from L.row0 of ``view``)."""
        torch = _arrays._torch()
        if prod == "hillshade":
            sp = S.make_params(azimuth=self.cfg.azimuth, altitude=self.cfg.altitude, pixel_size=L.pixel_size_m(),
                               nodata=self.nodata)
            return [PL.stencil_plan(view, tiles, sp, {S.OUTPUT_INDEX["hillshade"]: S.make_plane(out)}, keep=[out])]
        if prod == "openness":
            op = OP.make_params(max_distance=self.cfg.openness_distance, num_directions=self.cfg.openness_directions,
                                pixel_size=L.pixel_size_m(), sampling="reference", nodata=self.nodata)
            return [PL.openness_plan(view, tiles, op, None, out, keep=[out])]
        # topousm_fast: the level's large-radius coarse field and global scale, then the small radii per tile
        radii, weights = list(self.cfg.topousm_radii), self._topousm_weights()
        tile = max(t.core_h for t in tiles) if tiles else 4096
        thr = TU.topousm_fast_default_large_radius_threshold(int(tile))
        sr, sw, lr, lw = TU.split_radii_by_threshold(radii, weights, thr)
        lv = self.pyr.level_view(L) if level_raster is None else level_raster
        px = L.pixel_size_m()
        coarse = None
        keep = [out]
        if lr:
            scale = max(L.w / 2048.0, L.h / 2048.0, 1.0)
            ow, oh = max(1, int(round(L.w / scale))), max(1, int(round(L.h / scale)))
            cdem = TU.overview(lv, (oh, ow), nodata=self.nodata)
            coarse = TU.compute_topousm_fast_large_coarse_field(cdem, large_radii=lr, large_weights=lw,
                                                                 decimation=float(scale))
            keep.append(coarse)
        if stats is None:
            stats = global_stats_prepass(lv.contiguous(), "topousm_fast",
                                         {"radii": radii, "weights": weights, "pixel_size": px}, nodata=self.nodata)
        self.stats.setdefault(prod, []).append(float(stats[0]) if stats else None)
        # coordinates of the coarse field are the level's own (rows offset by the level's atlas row)
        tp, tkeep = TU.make_params(sr, sw, px, nodata=self.nodata, coarse=coarse, w_large=float(sum(lw)),
                                   full_shape=(L.h, L.w), scale=float(stats[0]) if stats else 0.0)
        keep += tkeep
        ltiles = []
        for t in tiles:  # topousm's field is sampled at level coordinates: the level is its own raster
            d = N.Tile()
            d.win_y0, d.win_x0, d.win_h, d.win_w = t.win_y0 - L.row0, t.win_x0, t.win_h, t.win_w
            d.core_y0, d.core_x0, d.core_h, d.core_w = t.core_y0 - L.row0, t.core_x0, t.core_h, t.core_w
            d.out_y0, d.out_x0 = t.out_y0, t.out_x0
            d.pixel_scale_x, d.pixel_scale_y = t.pixel_scale_x, t.pixel_scale_y
            ltiles.append(d)
        lview = _arrays.as_device_f32_2d(lv, name="level")
        return [PL.topousm_plan(lview, ltiles, tp, S.make_plane(out), keep=keep)]

    def _build(self, prod: str, sizes: Sequence[int]) -> None:
        out = self.outputs[prod]
        view = self.pyr.view
        n = 0
        n0 = len(self.plans)
        if prod == "topousm_fast":
            for L, ts in zip(self.pyr.levels, sizes):
                _, tiles = level_tiles(L, ts, self._padding(prod, ts))
                n += len(tiles)
                self.plans += self._level_plans(prod, L, tiles, out, view)
        else:
            tiles = []
            for L, ts in zip(self.pyr.levels, sizes):
                tiles += level_tiles(L, ts, self._padding(prod, ts))[1]
            n = len(tiles)
            # one plan over the tiles of every level (per-tile pixel scales carry the level)
            self.plans += self._level_plans(prod, self.pyr.levels[0], tiles, out, view)
        self.plan_products += [prod] * (len(self.plans) - n0)
        self.tile_counts[prod] = n

    # ------------------------------------------------------------ autotune
    def _tune(self, prod: str, L: Level, device_name: str) -> int:
        torch = _arrays._torch()
        cands = [c for c in self.cfg.candidates if c <= max(L.h, L.w)] or [min(self.cfg.candidates)]
        n = min(self.cfg.sample, L.h, L.w)
        key = Autotuner.key(device_name, prod, self.cfg.openness_distance if prod == "openness" else "",
                            tuple(self.cfg.topousm_radii) if prod == "topousm_fast" else "",
                            f"{L.h}x{L.w}", n)
        y0, x0 = (L.h - n) // 2, (L.w - n) // 2
        sub = self.pyr.atlas[L.row0 + y0:L.row0 + y0 + n, x0:x0 + n].contiguous()
        SL = Level(L.index, L.factor, 0, n, n, L.transform)
        sview = _arrays.as_device_f32_2d(sub, name="sample")
        out = torch.empty_like(sub)

        def measure(ts: int):
            _, tiles = level_tiles(SL, ts, self._padding(prod, ts))
            try:
                ps = self._level_plans(prod, SL, tiles, out, sview, stats=(1.0,), level_raster=sub)
            except N.FsgError:
                return None
            for p in ps:
                p.launch()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                for p in ps:
                    p.launch()
            e1.record()
            torch.cuda.synchronize()
            for p in ps:
                p.close()
            return e0.elapsed_time(e1) / 3.0 / (n * n)

        saved = self.stats.pop(prod, None)
        best = self.tuner.choose(key, cands, measure)
        if saved is not None:
            self.stats[prod] = saved
        else:
            self.stats.pop(prod, None)
        return best

    # ---------------------------------------------------------------- steps
    def step(self) -> None:
        for p in self.plans:
            p.launch()

    def capture(self) -> PL.GraphStep:
        self._graph = PL.GraphStep(self.step)
        return self._graph

    def replay(self) -> None:
        if self._graph is None:
            self.capture()
        self._graph.replay()

    def product_graph_ms(self, steps: int = 4) -> Dict[str, float]:
        """Device time of each product's share of the step: that product's plans captured
        into their own CUDA graph and replayed ``steps`` times (CUDA events around the
        replays on the current stream)."""
        torch = _arrays._torch()
        out = {}
        for prod in dict.fromkeys(self.plan_products):
            ps = [p for p, q in zip(self.plans, self.plan_products) if q == prod]
            g = PL.GraphStep(lambda ps=ps: [p.launch() for p in ps])
            g.replay()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(max(1, steps)):
                g.replay()
            e1.record()
            torch.cuda.synchronize()
            out[prod] = e0.elapsed_time(e1) / max(1, steps)
        return out

    def result(self) -> BatchResult:
        return BatchResult(self.outputs, dict(self.tile_sizes), dict(self.tile_counts), dict(self.stats))

    def close(self) -> None:
        self._graph = None
        for p in self.plans:
            p.close()
        self.plans = []


__all__ = ["Level", "Pyramid", "level_tiles", "BatchConfig", "BatchedTiles", "BatchResult", "PRODUCTS"]
