"""Pin the CPU oracle to golden vectors produced by the reference itself.

The fixtures in ``tests/golden`` were generated by ``tests/golden/make_golden.py``
from the reference's own block functions (CuPy -> NumPy, cupyx.scipy.ndimage ->
scipy.ndimage).  The oracle must reproduce them bit-exactly: it restates the
same float32 operation order with the same library calls.
"""
import json
import os

import numpy as np
import pytest

from oracle import restated as R


def _load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name + ".npz"))


def _meta(golden_dir, name):
    with open(os.path.join(golden_dir, name + ".json")) as f:
        return json.load(f)


def _eq(a, b):
    assert a.dtype == b.dtype, (a.dtype, b.dtype)
    assert a.shape == b.shape
    assert np.array_equal(a, b, equal_nan=True), float(np.nanmax(np.abs(a.astype(np.float64) - b)))


STENCIL_CASES = ["s1_fbm_10m", "s2_fbm_5m_nan", "s3_geo_edges_nan", "s4_tiny_3x5", "s5_single_valid",
                 "s6_all_nan", "s7_parabolic_cylinder", "s8_dome", "s9_big_void"]


@pytest.mark.parametrize("case", STENCIL_CASES)
def test_stencil_products_bit_exact(golden_dir, case):
    g = _load(golden_dir, "stencil")
    m = _meta(golden_dir, "stencil")[case]
    dem = g[f"{case}/dem"]
    kw = dict(pixel_size=m["pixel_size"], psx=m["psx"], psy=m["psy"])
    _eq(R.hillshade(dem.copy(), azimuth=m["azimuth"], altitude=m["altitude"], z_factor=m["z_factor"], **kw),
        g[f"{case}/hillshade"])
    for unit in ("degree", "percent", "radian"):
        _eq(R.slope(dem.copy(), unit=unit, **kw), g[f"{case}/slope_{unit}"])
    for ct in ("mean", "gaussian", "planform", "profile"):
        _eq(R.curvature(dem.copy(), curvature_type=ct, **kw), g[f"{case}/curvature_{ct}"])


def test_reference_curvature_known_answers(golden_dir):
    """tests/test_curvature_analytic.py:26-54 of the reference, on the oracle."""
    g = _load(golden_dir, "stencil")
    zero = 0.5 ** (1.0 / 2.2)
    cyl = g["s7_parabolic_cylinder/dem"]
    plan = R.curvature(cyl, curvature_type="planform")
    prof = R.curvature(cyl, curvature_type="profile")
    assert float(np.abs(plan[20:44, 20:44] - zero).max()) < 0.02
    assert float(np.abs(prof[20:44, 20:44] - zero).max()) > 0.05
    dome = g["s8_dome/dem"]
    for ct in ("planform", "profile"):
        assert float(np.abs(R.curvature(dome, curvature_type=ct)[20:44, 20:44] - zero).max()) > 0.05


@pytest.mark.parametrize("variant", ["clean", "nan"])
def test_spatial_smoothing_bit_exact(golden_dir, variant):
    g = _load(golden_dir, "smooth")
    dem = g[f"{variant}/dem"]
    for r, algo in ((1.0, "hillshade"), (4.0, "hillshade"), (16.0, "slope"), (40.0, "curvature"),
                    (100.0, "hillshade")):
        _eq(np.asarray(R.smooth_for_radius(dem.copy(), r, pixel_size=5.0, algorithm=algo), np.float32),
            g[f"{variant}/smooth_{algo}_{int(r)}"])


@pytest.mark.parametrize("variant", ["clean", "nan"])
def test_spatial_block_functions_bit_exact(golden_dir, variant):
    """compute_*_spatial_block and the multi-radius _direct_hillshade (smoothing + product)."""
    g = _load(golden_dir, "spatial")
    dem = g[f"{variant}/dem"]
    kw = dict(pixel_size=5.0, psx=5.0, psy=-5.0)
    for r in (1.0, 3.0, 12.0, 40.0):
        _eq(R.spatial_block(dem.copy(), "hillshade", r, azimuth=300.0, altitude=40.0, **kw),
            g[f"{variant}/hillshade_{int(r)}"])
        _eq(R.spatial_block(dem.copy(), "slope", r, **kw), g[f"{variant}/slope_{int(r)}"])
        _eq(R.spatial_block(dem.copy(), "curvature", r, curvature_type="profile", **kw),
            g[f"{variant}/curvature_profile_{int(r)}"])
    _eq(R.direct_multiscale(dem.copy(), "hillshade", [1, 4, 16], [0.5, 0.3, 0.2], **kw),
        g[f"{variant}/direct_hillshade_multiscale"])


def test_map_overlap_reflect_is_symmetric_padding():
    """dask's 'reflect' boundary repeats the edge sample; the depth is capped below the chunk."""
    b = np.arange(12, dtype=np.float32).reshape(3, 4)
    seen = {}

    def fn(x):
        seen["p"] = x.copy()
        return x

    out = R.map_overlap_reflect(fn, b, 2)
    assert np.array_equal(out, b)
    assert np.array_equal(seen["p"][2, :], np.array([1, 0, 0, 1, 2, 3, 3, 2], np.float32))
    R.map_overlap_reflect(fn, b, 50)
    assert seen["p"].shape == (3 + 4, 4 + 4)


@pytest.mark.parametrize("case", ["t1_clean", "t2_nan", "t3_halfmetre", "t4_nan_r2"])
def test_topousm_block_bit_exact(golden_dir, case):
    g = _load(golden_dir, "topousm")
    m = _meta(golden_dir, "topousm")[case]
    out = R.topousm_block(g[f"{case}/dem"].copy(), radii=[int(r) for r in g[f"{case}/radii"]],
                          weights=[float(w) for w in g[f"{case}/weights"]], pixel_size=m["pixel_size"])
    _eq(out, g[f"{case}/out"])


def test_down_up_sampling_bit_exact(golden_dir):
    g = _load(golden_dir, "topousm")
    dem = g["down/dem"]
    for f in (2, 4, 8):
        small = R.downsample_nan_aware(dem.copy(), f)
        _eq(small, g[f"down/f{f}"])
        _eq(R.upsample_to_shape(small, dem.shape), g[f"down/up{f}"])


def test_coarse_field_and_global_sampling_bit_exact(golden_dir):
    g = _load(golden_dir, "topousm")
    field = R.coarse_field(g["coarse/dem"].copy(), large_radii=[512, 2048],
                           large_weights=[2.0 / 63.0, 1.0 / 63.0], decimation=16.0)
    _eq(field, g["coarse/field"])
    _eq(R.bilinear_sample_coarse(field, 100, 180, 333, 433, 1024, 1280), g["coarse/sample"])
    _eq(R.bilinear_sample_coarse(field, 0, 40, 1240, 1280, 1024, 1280), g["coarse/sample_edge"])


def test_normalisation_statistics(golden_dir):
    g = _load(golden_dir, "topousm")
    assert R.topousm_scale(g["stats/outliers"])[0] == float(g["stats/outliers_scale"][0])
    assert R.topousm_scale(g["stats/ridge"])[0] == float(g["stats/ridge_scale"][0])
    # reference tests/test_topousm_fast_normalization.py:6-32 known answers
    assert 0.0 < R.topousm_scale(g["stats/outliers"])[0] < 0.2
    assert R.topousm_scale(g["stats/ridge"])[0] == pytest.approx(0.5, rel=1e-2)
    t2 = g["t2_nan/out"]
    s = R.topousm_scale(t2)
    assert s[0] == float(g["stats/t2_scale"][0])
    _eq(R.topousm_normalize(t2.copy(), s), g["stats/t2_norm"])
    st = R.stretch_stats(g["stats/stretch_in"])
    assert st == tuple(float(x) for x in g["stats/stretch"])


def test_topousm_norm_is_linear_without_clip():
    """reference tests/test_topousm_fast_normalization.py:35-44."""
    d = np.asarray([-4.0, -1.0, 0.0, 1.0, 4.0], np.float32)
    assert R.topousm_normalize(d, (2.0,)).tolist() == pytest.approx([-2.0, -0.5, 0.0, 0.5, 2.0])


OPEN_CASES = ["o1_fbm_nan", "o2_peak", "o2_pit", "o2_flat", "o3_aniso_d5", "o4_r256"]


@pytest.mark.parametrize("case", OPEN_CASES)
def test_openness_bit_exact(golden_dir, case):
    g = _load(golden_dir, "openness")
    m = _meta(golden_dir, "openness")[case]
    for ot in ("positive", "negative"):
        out = R.openness(g[f"{case}/dem"].copy(), openness_type=ot, num_directions=m["num_directions"],
                         max_distance=m["max_distance"], pixel_size=m["pixel_size"], psx=m["psx"], psy=m["psy"])
        _eq(out, g[f"{case}/{ot}"])


AO_CASES = ["a1_fbm_nan", "a2_aniso", "a3_r1", "a4_peak_pit", "a5_wide_radius", "a6_flat"]


@pytest.mark.parametrize("case", AO_CASES)
def test_ambient_occlusion_bit_exact(golden_dir, case):
    """compute_ambient_occlusion_block (_impl_ambient_occlusion.py:32-121): non-integer and
    unit radii, anisotropic scales, clamped (steep) and zero (flat) occlusion, NaN cells."""
    g = _load(golden_dir, "ambient_occlusion")
    m = _meta(golden_dir, "ambient_occlusion")[case]
    out = R.ambient_occlusion(g[f"{case}/dem"].copy(), num_samples=m["num_samples"], radius=m["radius"],
                              intensity=m["intensity"], pixel_size=m["pixel_size"], psx=m["psx"], psy=m["psy"])
    _eq(out, g[f"{case}/ao"])


def test_ambient_occlusion_stretch_and_spatial_bit_exact(golden_dir):
    """_direct_ambient_occlusion's display stretch (tile/dask_bridge.py:190-203) and
    compute_ambient_occlusion_spatial_block (_impl_ambient_occlusion.py:124-157) at
    decimation factors 1, 2 and 4, with and without NoData."""
    g = _load(golden_dir, "ambient_occlusion")
    a = R.ambient_occlusion(g["a1_fbm_nan/dem"].copy(), num_samples=16, radius=10.0, pixel_size=5.0, psx=5.0,
                            psy=-5.0)
    _eq(R.apply_stretch(a, (0.55, 0.4)), g["a1_fbm_nan/direct_stretch"])
    for dn in ("clean", "nan"):
        dem = g[f"spatial_{dn}/dem"]
        for r in (8, 40, 100):
            _eq(R.ambient_occlusion_spatial_block(dem.copy(), num_samples=16, radius=float(r), pixel_size=5.0,
                                                  psx=5.0, psy=-5.0), g[f"spatial_{dn}/ao_{r}"])
    assert [R.downsample_factor(r, pixel_size=5.0, algorithm="ambient_occlusion") for r in (8, 40, 100)] == [1, 2, 4]


@pytest.mark.parametrize("variant", ["clean", "nan"])
def test_openness_spatial_pieces_bit_exact(golden_dir, variant):
    """_downsample_nan_aware (block mean, enclosed voids filled, exterior kept NaN),
    _upsample_to_shape (NaN-aware zoom, odd target) and compute_openness_spatial_block at
    decimation factors 1, 2, 4 and 8."""
    g = _load(golden_dir, "openness_spatial")
    dem = g[f"{variant}/dem"]
    for f in (2, 4, 8):
        _eq(R.downsample_nan_aware(dem.copy(), f), g[f"{variant}/down_{f}"])
    small = g[f"{variant}/down_4"]
    _eq(R.upsample_to_shape(small, dem.shape), g[f"{variant}/up_4"])
    _eq(R.upsample_to_shape(small, (131, 97)), g[f"{variant}/up_4_odd"])
    for md in (12, 40, 80, 150):
        for ot in ("positive", "negative"):
            _eq(R.openness_spatial_block(dem.copy(), openness_type=ot, max_distance=md, pixel_size=5.0, psx=5.0,
                                         psy=-5.0), g[f"{variant}/openness_{ot}_{md}"])
    if variant == "nan":
        # the exterior strip keeps its NaN coarse cells; some empty interior cells are filled
        assert np.isnan(g["nan/down_8"][:, :2]).all()
        empty = np.isnan(dem).reshape(30, 4, 34, 4).all(axis=(1, 3))
        assert np.isnan(g["nan/down_4"][:, 5:]).sum() < empty[:, 5:].sum()


def test_spatial_combination_modes():
    """_combine_multiscale_dask / the hillshade branch: max / min propagate NaN, 'sum' and the
    plain mean add in order, invalid weights fall back to the plain mean."""
    a = np.asarray([[1.0, np.nan, 3.0]], np.float32)
    b = np.asarray([[2.0, 5.0, 1.0]], np.float32)
    c = np.asarray([[0.5, 1.0, 7.0]], np.float32)
    rs = [a, b, c]
    assert np.array_equal(R.combine_responses(rs, None, "slope", "max"), np.asarray([[2.0, np.nan, 7.0]], np.float32),
                          equal_nan=True)
    assert np.array_equal(R.combine_responses(rs, None, "openness", "min"),
                          np.asarray([[0.5, np.nan, 1.0]], np.float32), equal_nan=True)
    assert np.array_equal(R.combine_responses(rs, None, "curvature", "sum"), (a + b) + c, equal_nan=True)
    mean = ((a + b) + c) / np.float32(3)
    assert np.array_equal(R.combine_responses(rs, [1, -1, float("nan")] * 0 + [0, 0, 0], "slope"), mean,
                          equal_nan=True)
    assert np.array_equal(R.combine_responses(rs, [1, 2], "hillshade"), mean, equal_nan=True)
    assert np.array_equal(R.combine_responses([a], [3.0], "openness", "max"), a, equal_nan=True)


def test_openness_reference_known_answers(golden_dir):
    """reference tests/test_openness_yokoyama.py:1-47 on the oracle."""
    g = _load(golden_dir, "openness")
    c = 50

    def run(n, ot):
        return R.openness(g[f"{n}/dem"], openness_type=ot, num_directions=16, max_distance=40)[c, c]

    assert run("o2_peak", "positive") > run("o2_pit", "positive")
    assert run("o2_pit", "negative") > run("o2_peak", "negative")
    assert run("o2_flat", "positive") == pytest.approx(1.0, abs=1e-3)
    assert run("o2_flat", "negative") == pytest.approx(1.0, abs=1e-3)


def test_openness_r256_distances():
    assert R.openness_distances(256).tolist() == [25, 51, 76, 102, 128, 153, 179, 204, 230, 256]
    assert R.openness_distances(5).tolist() == [1, 2, 3, 4, 5]


def test_quantize_bit_exact(golden_dir):
    g = _load(golden_dir, "encoding")
    with open(os.path.join(golden_dir, "tables.json")) as f:
        t = json.load(f)
    qin = g["q/in"]
    for key, qp_ref in t["quantize_params"].items():
        algo, dt = key.split("/")
        if algo == "slope_radian":
            rng = R.resolve_output_range("slope", params={"unit": "radian"})
        else:
            rng = R.resolve_output_range(algo, params={})
        qp = R.quantize_params(rng[0], rng[1], dt)
        for k, v in qp_ref.items():
            assert qp[k] == v, (key, k)
        _eq(R.quantize_array(qin, qp, dt), g[f"q/{key}"])


def test_logic_tables(golden_dir):
    with open(os.path.join(golden_dir, "tables.json")) as f:
        t = json.load(f)
    for r, px, algo, f_ in t["downsample_factor"]:
        assert R.downsample_factor(r, pixel_size=px, algorithm=algo) == f_, (r, px, algo)
    for s, radii in t["auto_radii"]:
        assert R.auto_spatial_radii(s) == radii
    for n, w in t["auto_weights"]:
        assert R.auto_spatial_weights(n) == w
    for lat, mpd in t["meters_per_degree"]:
        assert list(R.meters_per_degree(lat)) == mpd
    for r, w, out in t["dedup"]:
        got = R.dedup_radii_weights(r, w)
        assert [got[0], got[1]] == out
    for r, w, out in t["resolve_radii_weights"]:
        got = R.resolve_spatial_radii_weights(r, w, 10.0, 3000)
        assert [list(got[0]), list(got[1])] == out
    for r, w, thr, out in t["split_radii"]:
        assert [list(x) for x in R.split_radii_by_threshold(r, w, thr)] == out
    for mr, mw, px, out in t["topousm_radii_norm"]:
        got = R.normalize_topousm_radii(mr, mw, px)
        assert [None if x is None else list(x) for x in got] == out


def test_tile_grid_clips_at_raster_edges():
    tiles = R.tile_grid(10000, 9000, 4096, 160)
    assert len(tiles) == 3 * 3
    ty, tx, cx, cy, cw, ch, wx, wy, ww, wh = tiles[0]
    assert (cx, cy, cw, ch, wx, wy, ww, wh) == (0, 0, 4096, 4096, 0, 0, 4256, 4256)
    ty, tx, cx, cy, cw, ch, wx, wy, ww, wh = tiles[4]
    assert (cx, cy, cw, ch, wx, wy, ww, wh) == (4096, 4096, 4096, 4096, 3936, 3936, 4416, 4416)
    ty, tx, cx, cy, cw, ch, wx, wy, ww, wh = tiles[-1]
    assert (cx, cy, cw, ch) == (8192, 8192, 808, 1808)
    assert (wx, wy, ww, wh) == (8032, 8032, 968, 1968)


def test_nodata_mask_merges_nan_and_sentinel():
    """core/tile_processor.py:185-196; reference tests/test_audit_p1_regressions.py:20-43."""
    d = np.asarray([[-9999.0, -9999.0000005, 1.0, np.nan], [-9998.99, 0.0, 2.0, 3.0]], np.float32)
    m = R.nodata_mask(d, -9999.0)
    assert m.tolist() == [[True, True, False, True], [False, False, False, False]]
    assert R.nodata_mask(d, float("nan")).tolist() == np.isnan(d).tolist()
    assert R.nodata_mask(d, None) is None


PP_CASES = ["pp1", "pp2_wide", "pp3_sparse", "pp4_all_valid", "pp5_none_valid"]


@pytest.mark.parametrize("case", PP_CASES)
def test_pushpull_fill_bit_exact(golden_dir, case):
    """pushpull_fill (_pyramid_fill.py:24-84): voids with an exterior strip, a wide void in a
    3-row grid (the apex collapses the long axis), sparse support, all / no valid cells."""
    g = _load(golden_dir, "prepare")
    _eq(R.pushpull_fill(g[f"{case}/coarse"], g[f"{case}/valid"]), g[f"{case}/filled"])


def test_prepare_pieces_bit_exact(golden_dir):
    """_nan_aware_coarse_average (declared mask + sentinels), _detect_sentinel_nodata /
    _detect_border_nodata (frame, spread sentinel, range extreme, mid-range spike, clean),
    _coarse_shape, _edge_connected_mask, _sample_coarse and _apply_band_fill
    (io/dem_preprocess.py:135-275, 729-826; utils/nodata_handler.py:13-25)."""
    g = _load(golden_dir, "prepare")
    m = _meta(golden_dir, "prepare")
    co, cm = R.nan_aware_coarse_average(g["avg/sample"], g["avg/declared"], 12, 16, None, [-9999.0, 0.0])
    _eq(co, g["avg/coarse"])
    assert np.array_equal(cm, g["avg/void"])
    for n, (sent, border) in m["detect"].items():
        a = g[f"det_{n}/sample"]
        v = np.isfinite(a)
        assert R.detect_sentinel_nodata(a, v) == sent, n
        assert R.detect_border_nodata(a, v) == border, n
    for w, h, cmax, ref in m["coarse_shape"]:
        assert list(R.coarse_shape(w, h, cmax)) == ref
    assert np.array_equal(R.edge_connected_mask(g["edge/mask"]), g["edge/connected"])
    b = m["band"]
    full = g["band/full"]
    H, W = full.shape
    band = full[b["row_off"]:b["row_off"] + b["bh"]]
    for mode, out_nd in (("enclosed", float("nan")), ("all", None)):
        out = R.apply_band_fill(band, np.zeros(band.shape, bool), row_off=b["row_off"], width=W, height=H,
                                ch=b["ch"], cw=b["cw"], do_fill=True, surface=g["band/surface"],
                                exterior=g["band/exterior"] if mode == "enclosed" else None,
                                extra_nodata=[-9999.0], fill_mode=mode, out_nodata=out_nd)
        _eq(out, g[f"band/{mode}"])
    fv, ex = R.sample_coarse_band(g["band/surface"], g["band/exterior"], b["row_off"], b["bh"], W, H, b["ch"],
                                  b["cw"])
    _eq(fv, g["band/sample_vals"])
    assert np.array_equal(ex, g["band/sample_ext"])
