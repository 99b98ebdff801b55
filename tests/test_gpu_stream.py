"""The streaming tile loop (core/stream.py: process_raster_tiles) over the
reader / writer interface equals the in-memory tile loop (process_dem_array) on
the same raster: local-mode products and openness bit for bit (same windows,
same statistics), topousm_fast within float rounding of the overview (the
reader averages it in float64, the device overview kernel in float-float)."""
import numpy as np
import pytest

from tests._parity import assert_same_nan, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300.core import stream, tile_loop
    from fujishadergpu_gb300.io import tile_io
    return stream, tile_loop, tile_io


def _dem(h, w, seed, sentinel=None):
    from fujishadergpu_gb300 import synth
    d = synth.fbm_ridged(h, w, hurst=0.8, seed_fbm=seed, seed_ridged=seed + 1, lo=0.0, hi=3000.0)
    d[synth.nodata_disks(h, w, count=4, seed=seed + 2, rmin=5.0, rmax=25.0)] = np.nan if sentinel is None else sentinel
    return d


@pytest.mark.parametrize("algorithm,kw,dtype", [
    ("hillshade", dict(mode="local"), "uint8"),
    ("curvature", dict(mode="local", curvature_type="planform"), "float32"),
    ("openness", dict(mode="local", max_distance=30), "float32"),
    ("ambient_occlusion", dict(mode="local", radius=8.0), "uint8"),
])
def test_streamed_local_products_equal_the_in_memory_loop(mods, algorithm, kw, dtype):
    stream, tile_loop, tile_io = mods
    dem = _dem(700, 810, 141, sentinel=-9999.0)
    common = dict(tile_size=256, pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0, output_dtype=dtype, **kw)
    ref = tile_loop.process_dem_array(torch.from_numpy(dem).cuda(), algorithm, nodata=-9999.0, **common)
    w = tile_io.ArrayWriter(dem.shape, dtype)
    res = stream.process_raster_tiles(tile_io.ArrayReader(dem, nodata=-9999.0), w, algorithm, band_tiles=1, **common)
    assert res.bands == 3 and res.tiles == ref.tiles and res.padding == ref.padding
    if ref.stats is not None:
        assert tuple(res.stats) == tuple(ref.stats)
    assert np.array_equal(w.data, to_np(ref.output), equal_nan=True)


def test_streamed_topousm_from_raw_files(mods, tmp_path):
    stream, tile_loop, tile_io = mods
    dem = _dem(1100, 900, 151)
    src = str(tmp_path / "dem.f32")
    tile_io.write_raw(src, dem)
    dst = str(tmp_path / "topousm.f32")
    common = dict(tile_size=256, pixel_size=10.0, pixel_scale_x=10.0, pixel_scale_y=-10.0,
                  radii=[2, 8, 32, 128, 512], weights=[16 / 31, 8 / 31, 4 / 31, 2 / 31, 1 / 31])
    ref = tile_loop.process_dem_array(torch.from_numpy(dem).cuda(), "topousm_fast", **common)
    w = tile_io.RawWriter(dst, dem.shape, "float32")
    res = stream.process_raster_tiles(tile_io.RawReader(src), w, "topousm_fast", band_tiles=2, **common)
    w.close()
    got = tile_io.RawReader(dst).read_window(0, 0, *dem.shape)
    r = to_np(ref.output)
    assert res.stats[0] == pytest.approx(ref.stats[0], rel=1e-6)
    assert_same_nan(got, r, "streamed topousm")
    m = ~np.isnan(r)
    assert float(np.abs(got[m].astype(np.float64) - r[m]).max()) <= 1e-5 * 2 * 1.176


def test_streamed_geographic_slope(mods):
    stream, tile_loop, tile_io = mods
    dem = _dem(520, 600, 161)
    tr = (1.0 / 3600.0, 0.0, 135.0, 0.0, -(45.0 - 30.0) / 520, 45.0)
    common = dict(tile_size=128, mode="local", geographic=True, pixel_size=1.0)
    ref = tile_loop.process_dem_array(torch.from_numpy(dem).cuda(), "slope", transform=tr, **common)
    w = tile_io.ArrayWriter(dem.shape)
    stream.process_raster_tiles(tile_io.ArrayReader(dem, transform=tr), w, "slope", band_tiles=3, **common)
    assert np.array_equal(w.data, to_np(ref.output), equal_nan=True)


def test_streaming_rejects_spatial_mode(mods):
    stream, _, tile_io = mods
    dem = _dem(64, 64, 171)
    with pytest.raises(ValueError, match="spatial mode"):
        stream.process_raster_tiles(tile_io.ArrayReader(dem), tile_io.ArrayWriter(dem.shape), "hillshade",
                                    mode="spatial", radii=[2, 4])
