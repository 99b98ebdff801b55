"""Host logic of the batched uneven-tile workload: per-level tile grids in
atlas coordinates (windows clipped at each level's edges, per-tile geographic
pixel scales, core/tile_processor.py:910-932 and :1610-1627) and the tile-shape
autotuner's choice and cache."""
import json

import pytest

from fujishadergpu_gb300.core.autotune import Autotuner
from fujishadergpu_gb300.core.batch import Level, level_tiles
from fujishadergpu_gb300.io.raster_info import tile_pixel_scales


def _level(index, row0, h, w):
    f = 1 << index
    return Level(index, f, row0, h, w, (f / 3600.0, 0.0, 135.0, 0.0, -f * 15.0 / 4096.0, 45.0))


@pytest.mark.parametrize("index,row0,h,w,tile,pad", [(0, 0, 4096, 8192, 1024, 64), (1, 4096, 2048, 4096, 512, 40),
                                                     (2, 6144, 1024, 2048, 256, 288), (2, 6144, 1000, 1900, 256, 8)])
def test_level_tiles_cover_the_level_once(index, row0, h, w, tile, pad):
    L = _level(index, row0, h, w)
    infos, tiles = level_tiles(L, tile, pad)
    covered = set()
    for info, t in zip(infos, tiles):
        # windows clipped at the level's own edges, in atlas rows
        assert row0 <= t.win_y0 and t.win_y0 + t.win_h <= row0 + h
        assert 0 <= t.win_x0 and t.win_x0 + t.win_w <= w
        assert t.win_y0 <= t.core_y0 and t.core_y0 + t.core_h <= t.win_y0 + t.win_h
        assert t.win_x0 <= t.core_x0 and t.core_x0 + t.core_w <= t.win_x0 + t.win_w
        assert (t.out_y0, t.out_x0) == (t.core_y0, t.core_x0)
        assert t.core_h <= tile and t.core_w <= tile
        # halo = pad where the level continues, clipped at its edges
        assert t.core_y0 - t.win_y0 == min(pad, t.core_y0 - row0)
        assert t.core_x0 - t.win_x0 == min(pad, t.core_x0)
        # per-tile metric scales at the tile core's latitude, in level coordinates
        assert (t.pixel_scale_x, t.pixel_scale_y) == tile_pixel_scales(info.core_y, info.core_h, L.transform)
        covered.add((t.core_y0, t.core_x0))
    ny, nx = -(-h // tile), -(-w // tile)
    assert len(covered) == len(tiles) == ny * nx
    assert sum(t.core_h * t.core_w for t in tiles) == h * w


def test_scales_follow_latitude_across_levels():
    L0, L2 = _level(0, 0, 4096, 4096), _level(2, 6144, 1024, 1024)
    _, t0 = level_tiles(L0, 1024, 8)
    _, t2 = level_tiles(L2, 256, 8)
    # southward (larger row) tiles have wider metre spacing in x; level 2 pixels are 4x level 0's
    assert t0[0].pixel_scale_x < t0[-1].pixel_scale_x
    assert t2[0].pixel_scale_x == pytest.approx(4 * t0[0].pixel_scale_x, rel=2e-3)
    assert t0[0].pixel_scale_y < 0 and t2[0].pixel_scale_y < 0


def test_autotuner_picks_the_cheapest_and_caches(tmp_path):
    path = str(tmp_path / "tune.json")
    calls = []

    def measure(c):
        calls.append(c)
        return {256: 3.0, 512: 1.5, 1024: 2.0, 2048: None}[c]

    t = Autotuner(path=path, enabled=True)
    k = Autotuner.key("GPU", "hillshade", "4096x4096")
    assert t.choose(k, [256, 512, 1024, 2048], measure) == 512
    assert calls == [256, 512, 1024, 2048]
    data = json.load(open(path))
    assert data[k]["choice"] == 512 and "2048" not in data[k]["costs"]
    # a fresh tuner reads the cache and measures nothing
    calls.clear()
    t2 = Autotuner(path=path, enabled=True)
    assert t2.choose(k, [256, 512, 1024], measure) == 512 and calls == []
    # a cached choice outside the candidates is re-measured
    assert t2.choose(k, [256, 1024], measure) == 1024
    # measuring disabled: the first candidate, nothing measured
    calls.clear()
    t3 = Autotuner(path=str(tmp_path / "none.json"), enabled=False)
    assert t3.choose(k, [1024, 256], measure) == 1024 and calls == []
