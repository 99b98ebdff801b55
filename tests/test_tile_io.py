"""Tile I/O behind the reader / writer interface (io/tile_io.py): in-memory and
raw-file rasters, window reads and writes, the averaged overview, the
reference's read_tile_window / write_tile_output shape (core/tile_io.py:49-72).
CPU only; the streaming tile loop over these readers is in test_gpu_stream.py."""
import numpy as np
import pytest

from fujishadergpu_gb300.io import tile_io as TI


def _raster(h=97, w=131, seed=0):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((h, w)).astype(np.float32) * 100 + 500
    a[10:20, 30:45] = np.nan
    a[50, 60] = -9999.0
    return a


def test_array_reader_windows_and_samples():
    a = _raster()
    r = TI.ArrayReader(a, nodata=-9999.0, transform=(1, 0, 0, 0, -1, 0))
    assert r.shape == a.shape and r.nodata == -9999.0 and r.transform == (1, 0, 0, 0, -1, 0)
    assert np.array_equal(r.read_window(5, 7, 20, 30), a[5:25, 7:37], equal_nan=True)
    rows, cols = np.array([0, 3, 96]), np.array([1, 130])
    assert np.array_equal(r.read_rows_cols(rows, cols), a[rows][:, cols], equal_nan=True)
    with pytest.raises(ValueError, match="outside"):
        r.read_window(90, 0, 10, 5)


@pytest.mark.parametrize("f", [1, 3, 8])
def test_overview_is_the_nan_aware_cell_mean(f):
    a = _raster(96, 120)
    r = TI.ArrayReader(a, nodata=-9999.0)
    oh, ow = 96 // f, 120 // f
    got = r.read_overview(oh, ow)
    cells = np.where(np.abs(a - np.float32(-9999.0)) <= 1e-6, np.nan, a).astype(np.float64)
    with np.errstate(invalid="ignore"), pytest.warns(RuntimeWarning) if f == 1 else _nullctx():
        ref = np.nanmean(cells.reshape(oh, f, ow, f), axis=(1, 3)).astype(np.float32)
    assert np.array_equal(got, ref, equal_nan=True)


class _nullctx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def test_overview_partition_for_uneven_factors():
    a = np.arange(7 * 10, dtype=np.float32).reshape(7, 10)
    got = TI.ArrayReader(a).read_overview(3, 4)
    rb, cb = TI._cell_bounds(7, 3), TI._cell_bounds(10, 4)
    for i in range(3):
        for j in range(4):
            assert got[i, j] == np.float32(a[rb[i]:rb[i + 1], cb[j]:cb[j + 1]].astype(np.float64).mean())
    # every pixel belongs to exactly one cell: [floor(i n / o), floor((i + 1) n / o))
    assert list(rb) == [0, 2, 4, 7] and list(cb) == [0, 2, 5, 7, 10]


def test_raw_file_round_trip(tmp_path):
    a = _raster()
    p = str(tmp_path / "dem.f32")
    TI.write_raw(p, a, nodata=-9999.0, transform=(10.0, 0.0, 5.0, 0.0, -10.0, 7.0))
    r = TI.RawReader(p)
    assert r.shape == a.shape and r.nodata == -9999.0 and r.transform == (10.0, 0.0, 5.0, 0.0, -10.0, 7.0)
    assert np.array_equal(r.read_window(0, 0, *a.shape), a, equal_nan=True)
    assert np.array_equal(r.read_overview(48, 65), TI.ArrayReader(a, nodata=-9999.0).read_overview(48, 65),
                          equal_nan=True)
    out = str(tmp_path / "out.u8")
    w = TI.RawWriter(out, a.shape, "uint8")
    w.write_window(3, 4, np.full((5, 6), 7, np.uint8))
    w.close()
    back = TI.RawReader(out)
    full = back.read_window(0, 0, *a.shape)
    assert full[3:8, 4:10].min() == 7 and full.sum() == 7 * 30


def test_tile_window_helpers_follow_the_tile_grid():
    from fujishadergpu_gb300.core.tile_loop import tile_grid
    a = _raster(300, 410)
    r = TI.ArrayReader(a)
    w = TI.ArrayWriter(a.shape)
    for t in tile_grid(300, 410, 128, 16):
        win = TI.read_tile_window(r, t)
        assert win.shape == (t.win_h, t.win_w)
        core = win[t.core_y - t.win_y:t.core_y - t.win_y + t.core_h, t.core_x - t.win_x:t.core_x - t.win_x + t.core_w]
        TI.write_tile_output(w, t, core)
    assert np.array_equal(w.data, a, equal_nan=True)
