"""Generate the golden fixtures in this folder from the reference's own code.

Run in a container that holds the reference sources, naming the folder that
contains its ``FujiShaderGPU`` package (or set ``FSG_REFERENCE_ROOT``)::

    python tests/golden/make_golden.py --reference <reference checkout>

It imports the reference's unmodified block functions through
``reference_shim`` (CuPy -> NumPy, cupyx.scipy.ndimage -> scipy.ndimage) and
saves inputs and outputs as ``.npz`` fixtures.  The fixtures are committed; the
tests read only them, never the reference.
"""
from __future__ import annotations

import json
import os
import sys

sys.dont_write_bytecode = True
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

import reference_shim  # noqa: E402
from fujishadergpu_gb300 import synth  # noqa: E402


SPATIAL_BLOCK_RADII = (1.0, 3.0, 12.0, 40.0)
OPENNESS_SPATIAL_FACTORS = (2, 4, 8)
OPENNESS_ODD_TARGET = (131, 97)
OPENNESS_SPATIAL_DISTANCES = (12, 40, 80, 150)   # decimation factors 1, 2, 4, 8 at 5 m


def _stub_rasterio():
    import types
    if "rasterio" not in sys.modules:
        sys.modules["rasterio"] = types.ModuleType("rasterio")


def _with_disks(dem, count, seed, rmin, rmax):
    m = synth.nodata_disks(dem.shape[0], dem.shape[1], count=count, seed=seed, rmin=rmin, rmax=rmax)
    out = dem.copy()
    out[m] = np.nan
    return out


def stencil_cases():
    cases = []
    d1 = synth.fbm(64, 96, hurst=0.8, seed=11, lo=0.0, hi=3000.0)
    cases.append(dict(name="s1_fbm_10m", dem=d1, psx=10.0, psy=-10.0, pixel_size=10.0,
                      azimuth=315.0, altitude=45.0, z_factor=1.0))
    d2 = _with_disks(synth.fbm(72, 90, hurst=0.7, seed=12, lo=0.0, hi=4000.0), 6, 13, 2.0, 9.0)
    cases.append(dict(name="s2_fbm_5m_nan", dem=d2, psx=5.0, psy=-5.0, pixel_size=5.0,
                      azimuth=200.0, altitude=30.0, z_factor=2.0))
    d3 = synth.fbm(40, 33, hurst=0.7, seed=14, lo=100.0, hi=900.0)
    d3[0:3, 5:9] = np.nan
    d3[-4:, -3:] = np.nan
    d3[17, 0] = np.nan
    d3[20:23, 14:16] = np.nan
    cases.append(dict(name="s3_geo_edges_nan", dem=d3, psx=26.8, psy=-30.8, pixel_size=28.8,
                      azimuth=315.0, altitude=45.0, z_factor=1.0))
    d4 = synth.fbm(3, 5, hurst=0.8, seed=15, lo=0.0, hi=50.0)
    cases.append(dict(name="s4_tiny_3x5", dem=d4, psx=1.0, psy=-1.0, pixel_size=1.0,
                      azimuth=315.0, altitude=45.0, z_factor=1.0))
    d5 = np.full((6, 7), np.nan, np.float32)
    d5[2, 3] = 10.0
    cases.append(dict(name="s5_single_valid", dem=d5, psx=2.0, psy=-2.0, pixel_size=2.0,
                      azimuth=315.0, altitude=45.0, z_factor=1.0))
    d6 = np.full((5, 5), np.nan, np.float32)
    cases.append(dict(name="s6_all_nan", dem=d6, psx=2.0, psy=-2.0, pixel_size=2.0,
                      azimuth=315.0, altitude=45.0, z_factor=1.0))
    x = np.arange(64, dtype=np.float32)[None, :].repeat(64, axis=0)
    cyl = (0.01 * (x - 32.0) ** 2).astype(np.float32)
    cases.append(dict(name="s7_parabolic_cylinder", dem=cyl, psx=None, psy=None, pixel_size=1.0,
                      azimuth=315.0, altitude=45.0, z_factor=1.0))
    y = np.arange(64, dtype=np.float32)[:, None].repeat(64, axis=1)
    dome = (-0.01 * ((x - 32.0) ** 2 + (y - 32.0) ** 2)).astype(np.float32)
    cases.append(dict(name="s8_dome", dem=dome, psx=None, psy=None, pixel_size=1.0,
                      azimuth=315.0, altitude=45.0, z_factor=1.0))
    d9 = synth.fbm(48, 52, hurst=0.8, seed=16, lo=0.0, hi=1500.0)
    d9[10:30, 20:40] = np.nan  # NaN block larger than the 4 px fill reach
    cases.append(dict(name="s9_big_void", dem=d9, psx=3.0, psy=3.0, pixel_size=3.0,
                      azimuth=90.0, altitude=60.0, z_factor=1.0))
    return cases


def main():
    ref = reference_shim.load()
    _stub_rasterio()
    import importlib
    raster_info = importlib.import_module("FujiShaderGPU.io.raster_info")
    tile_compute = importlib.import_module("FujiShaderGPU.core.tile_compute")

    hs_mod = ref._impl_hillshade
    sl_mod = ref._impl_slope
    cv_mod = ref._impl_curvature
    tu_mod = ref._impl_topousm_fast
    op_mod = ref._impl_openness
    nu = ref._nan_utils

    # ---------------------------------------------------------------- stencils
    meta = {}
    arrays = {}
    for c in stencil_cases():
        n = c["name"]
        dem = c["dem"]
        kw = dict(pixel_size=c["pixel_size"], pixel_scale_x=c["psx"], pixel_scale_y=c["psy"])
        arrays[f"{n}/dem"] = dem
        arrays[f"{n}/hillshade"] = hs_mod.compute_hillshade_block(
            dem.copy(), azimuth=c["azimuth"], altitude=c["altitude"], z_factor=c["z_factor"], **kw)
        for unit in ("degree", "percent", "radian"):
            arrays[f"{n}/slope_{unit}"] = sl_mod.compute_slope_block(dem.copy(), unit=unit, **kw)
        for ct in ("mean", "gaussian", "planform", "profile"):
            arrays[f"{n}/curvature_{ct}"] = cv_mod.compute_curvature_block(
                dem.copy(), curvature_type=ct, **kw)
        meta[n] = {k: c[k] for k in ("psx", "psy", "pixel_size", "azimuth", "altitude", "z_factor")}
    np.savez_compressed(os.path.join(HERE, "stencil.npz"), **arrays)
    with open(os.path.join(HERE, "stencil.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)

    # ------------------------------------------------------- spatial-mode smoothing
    arrays = {}
    meta = {}
    sm = synth.fbm(96, 112, hurst=0.8, seed=17, lo=0.0, hi=2000.0)
    sm_nan = _with_disks(sm, 4, 18, 3.0, 10.0)
    for dn, d in (("clean", sm), ("nan", sm_nan)):
        arrays[f"{dn}/dem"] = d
        for r, algo in ((1.0, "hillshade"), (4.0, "hillshade"), (16.0, "slope"), (40.0, "curvature"),
                        (100.0, "hillshade")):
            out = nu._smooth_for_radius(d.copy(), r, pixel_size=5.0, algorithm_name=algo)
            arrays[f"{dn}/smooth_{algo}_{int(r)}"] = np.asarray(out, np.float32)
    np.savez_compressed(os.path.join(HERE, "smooth.npz"), **arrays)

    # ------------------------------------------------ spatial-mode block functions
    arrays = {}
    sp = synth.fbm(80, 96, hurst=0.8, seed=19, lo=0.0, hi=2500.0)
    sp_nan = _with_disks(sp, 3, 20, 3.0, 8.0)
    for dn, d in (("clean", sp), ("nan", sp_nan)):
        arrays[f"{dn}/dem"] = d
        kw = dict(pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0)
        for r in SPATIAL_BLOCK_RADII:
            arrays[f"{dn}/hillshade_{int(r)}"] = hs_mod.compute_hillshade_spatial_block(
                d.copy(), radius=r, azimuth=300.0, altitude=40.0, **kw)
            arrays[f"{dn}/slope_{int(r)}"] = sl_mod.compute_slope_spatial_block(d.copy(), radius=r, **kw)
            # _curv_spatial (_impl_curvature.py:72-78) is a closure inside process(): the same two calls
            smc = nu._smooth_for_radius(d.copy(), r, pixel_size=5.0, algorithm_name="curvature")
            arrays[f"{dn}/curvature_profile_{int(r)}"] = cv_mod.compute_curvature_block(
                smc, curvature_type="profile", **kw)
        db = importlib.import_module("FujiShaderGPU.algorithms.tile.dask_bridge")
        arrays[f"{dn}/direct_hillshade_multiscale"] = db._direct_hillshade(
            d.copy(), dict(radii=[1, 4, 16], weights=[0.5, 0.3, 0.2], pixel_size=5.0,
                           pixel_scale_x=5.0, pixel_scale_y=-5.0))
    np.savez_compressed(os.path.join(HERE, "spatial.npz"), **arrays)

    # ------------------------------------------------- openness spatial-mode block
    arrays = {}
    ob = synth.fbm(120, 136, hurst=0.8, seed=23, lo=0.0, hi=2500.0)
    ob_nan = _with_disks(ob, 4, 24, 6.0, 14.0)
    ob_nan[:, :20] = np.nan  # exterior strip: border-connected coarse voids stay NaN
    for dn, d in (("clean", ob), ("nan", ob_nan)):
        arrays[f"{dn}/dem"] = d
        for f in OPENNESS_SPATIAL_FACTORS:
            arrays[f"{dn}/down_{f}"] = np.asarray(nu._downsample_nan_aware(d.copy(), f), np.float32)
        small = arrays[f"{dn}/down_4"]
        arrays[f"{dn}/up_4"] = np.asarray(nu._upsample_to_shape(small, d.shape), np.float32)
        arrays[f"{dn}/up_4_odd"] = np.asarray(nu._upsample_to_shape(small, OPENNESS_ODD_TARGET), np.float32)
        for md in OPENNESS_SPATIAL_DISTANCES:
            for ot in ("positive", "negative"):
                arrays[f"{dn}/openness_{ot}_{md}"] = op_mod.compute_openness_spatial_block(
                    d.copy(), openness_type=ot, num_directions=16, max_distance=md, pixel_size=5.0,
                    pixel_scale_x=5.0, pixel_scale_y=-5.0)
    np.savez_compressed(os.path.join(HERE, "openness_spatial.npz"), **arrays)

    # ---------------------------------------------------------------- topousm
    arrays = {}
    meta = {}
    t1 = synth.fbm(160, 200, hurst=0.8, seed=21, lo=0.0, hi=3500.0)
    t2 = _with_disks(t1, 5, 22, 3.0, 25.0)
    t2[:, :6] = np.nan  # exterior strip touching the window edge
    tcases = [
        ("t1_clean", t1, [1, 2, 8, 32, 64, 128], [32, 16, 8, 4, 2, 1], 10.0),
        ("t2_nan", t2, [1, 2, 8, 32, 64, 128], [32, 16, 8, 4, 2, 1], 10.0),
        ("t3_halfmetre", t1[:90, :77].copy(), [4, 16, 48], [0.5, 0.3, 0.2], 0.5),
        ("t4_nan_r2", t2[:50, :61].copy(), [2], [1.0], 5.0),
    ]
    for n, d, radii, w, px in tcases:
        wsum = float(sum(w))
        wn = [float(x) / wsum for x in w]
        arrays[f"{n}/dem"] = d
        arrays[f"{n}/radii"] = np.asarray(radii, np.int64)
        arrays[f"{n}/weights"] = np.asarray(wn, np.float64)
        arrays[f"{n}/out"] = tu_mod.compute_topousm_fast_efficient_block(
            d.copy(), radii=radii, weights=wn, pixel_size=px)
        meta[n] = {"pixel_size": px}
    # down/up-sampling helpers on their own
    du = _with_disks(synth.fbm(70, 93, hurst=0.7, seed=23, lo=0.0, hi=1000.0), 3, 24, 4.0, 14.0)
    du[:, :9] = np.nan
    arrays["down/dem"] = du
    for f in (2, 4, 8):
        small = nu._downsample_nan_aware(du.copy(), f)
        arrays[f"down/f{f}"] = small
        arrays[f"down/up{f}"] = nu._upsample_to_shape(small, du.shape)
    # coarse large-radius field + bilinear sample at global coordinates
    cdem = _with_disks(synth.fbm(64, 80, hurst=0.8, seed=25, lo=0.0, hi=3500.0), 2, 26, 2.0, 5.0)
    field = tu_mod.compute_topousm_fast_large_coarse_field(
        cdem, large_radii=[512, 2048], large_weights=[2.0 / 63.0, 1.0 / 63.0], decimation=16.0)
    arrays["coarse/dem"] = cdem
    arrays["coarse/field"] = field
    arrays["coarse/sample"] = nu._bilinear_sample_coarse(field, 100, 180, 333, 433, 1024, 1280)
    arrays["coarse/sample_edge"] = nu._bilinear_sample_coarse(field, 0, 40, 1240, 1280, 1024, 1280)
    # normalisation statistics
    rng = np.random.default_rng(27)
    base = rng.normal(0.0, 0.01, size=(2048,)).astype(np.float32)
    base[:3] = np.asarray([10.0, -8.0, 12.0], np.float32)
    arrays["stats/outliers"] = base
    arrays["stats/outliers_scale"] = np.asarray(ref._normalization.topousm_fast_stat_func(base), np.float64)
    ridge = np.concatenate([np.full((800,), 0.01, np.float32), np.full((200,), 0.5, np.float32)])
    arrays["stats/ridge"] = ridge
    arrays["stats/ridge_scale"] = np.asarray(ref._normalization.topousm_fast_stat_func(ridge), np.float64)
    tout = arrays["t2_nan/out"]
    arrays["stats/t2_scale"] = np.asarray(ref._normalization.topousm_fast_stat_func(tout), np.float64)
    arrays["stats/t2_norm"] = ref._global_stats.apply_global_normalization(
        tout.copy(), ref._normalization.topousm_fast_norm_func,
        ref._normalization.topousm_fast_stat_func(tout))
    vals = rng.random(5000).astype(np.float32) ** 3
    vals[::97] = np.nan
    arrays["stats/stretch_in"] = vals
    arrays["stats/stretch"] = np.asarray(ref._global_stats.robust_unsigned_stretch_stat_func(vals), np.float64)
    np.savez_compressed(os.path.join(HERE, "topousm.npz"), **arrays)
    with open(os.path.join(HERE, "topousm.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)

    # ---------------------------------------------------------------- openness
    arrays = {}
    meta = {}
    o1 = _with_disks(synth.fbm(96, 96, hurst=0.7, seed=31, lo=0.0, hi=800.0), 3, 32, 2.0, 8.0)
    yy, xx = np.mgrid[0:101, 0:101]
    rad = np.sqrt((xx - 50) ** 2 + (yy - 50) ** 2)
    o4 = synth.fbm_ridged(320, 320, hurst=0.7, seed_fbm=35, seed_ridged=36, lo=0.0, hi=1200.0)
    ocases = [
        ("o1_fbm_nan", o1, 16, 20, 5.0, 5.0, -5.0),
        ("o2_peak", (50 - rad).astype(np.float32), 16, 40, 1.0, None, None),
        ("o2_pit", (rad - 50).astype(np.float32), 16, 40, 1.0, None, None),
        ("o2_flat", np.zeros((101, 101), np.float32), 16, 40, 1.0, None, None),
        ("o3_aniso_d5", o1[:40, :50].copy(), 8, 5, 4.0, 3.0, -5.0),
        ("o4_r256", o4, 16, 256, 5.0, 5.0, -5.0),
    ]
    for n, d, nd, md, px, psx, psy in ocases:
        arrays[f"{n}/dem"] = d
        for ot in ("positive", "negative"):
            arrays[f"{n}/{ot}"] = op_mod.compute_openness_vectorized(
                d.copy(), openness_type=ot, num_directions=nd, max_distance=md,
                pixel_size=px, pixel_scale_x=psx, pixel_scale_y=psy)
        meta[n] = {"num_directions": nd, "max_distance": md, "pixel_size": px,
                   "psx": psx, "psy": psy}
    np.savez_compressed(os.path.join(HERE, "openness.npz"), **arrays)
    with open(os.path.join(HERE, "openness.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)

    # ---------------------------------------------------------------- encoding + tables
    oe = ref.output_encoding
    enc = {}
    for algo in ("hillshade", "slope", "curvature", "openness", "topousm_fast"):
        rng_ = oe.resolve_output_range(algo, params={})
        for dt in ("uint8", "int16"):
            enc[f"{algo}/{dt}"] = oe.quantize_params(rng_[0], rng_[1], dt)
    enc["slope_radian/uint8"] = oe.quantize_params(*oe.resolve_output_range("slope", params={"unit": "radian"}), "uint8")
    qin = np.concatenate([
        np.linspace(-1.5, 1.5, 301, dtype=np.float32),
        np.asarray([np.nan, np.inf, -np.inf, 0.5, -0.5, 1.176, -1.176], np.float32),
        np.linspace(0.0, 90.0, 181, dtype=np.float32),
    ])
    arrays = {"q/in": qin}
    for key, qp in enc.items():
        arrays[f"q/{key}"] = oe.quantize_array(qin, qp, key.split("/")[1])
    tables = {"quantize_params": enc}
    tables["downsample_factor"] = [
        [r, px, algo, nu._radius_to_downsample_factor(r, pixel_size=px, algorithm_name=algo)]
        for algo in ("topousm_fast", "hillshade", "slope", "curvature", "openness")
        for px in (0.25, 0.5, 1.0, 5.0, 10.0, 30.0)
        for r in (1, 2, 4, 8, 16, 24, 28, 32, 48, 64, 100, 128, 256, 512, 1024, 2048)
    ]
    sp = ref.spatial_mode
    tables["auto_radii"] = [[s, sp.auto_spatial_radii(s)] for s in (10, 19, 20, 79, 80, 319, 320, 1279, 1280,
                                                                     5119, 5120, 20479, 20480, 40000, 65536)]
    tables["auto_weights"] = [[n, sp.auto_spatial_weights(n)] for n in range(0, 7)]
    tables["meters_per_degree"] = [[lat, list(raster_info.meters_per_degree(lat))]
                                   for lat in (0.0, 15.0, 30.0, 35.5, 37.5, 40.0, 45.0, 60.0, 89.9)]
    tables["dedup"] = [
        [r, w, list(tile_compute.deduplicate_radii_weights(r, w))]
        for r, w in (([2, 8, 8, 32], [0.4, 0.3, 0.2, 0.1]), ([4, 4], None), ([1, 2], [1.0, -1.0]),
                     ([2, 8], [0.0, 0.0]), ([16, 2, 16], [1, 2, 3]))
    ]
    tables["resolve_radii_weights"] = [
        [r, w, [list(x) if x is not None else None for x in nu._resolve_spatial_radii_weights(r, w, 10.0, 3000)]]
        for r, w in ((None, None), ([4, 16.4, 64], None), ([4, 16, 64], [3, 2, 1]), ([4, 16], [0, 0]),
                     ([-1, 0], None), ([8, 8, 2], [1, 1, 1]))
    ]
    tables["split_radii"] = [
        [r, w, thr, [list(x) for x in tu_mod.split_radii_by_threshold(r, w, thr)]]
        for r, w, thr in (([2, 8, 32, 128, 512, 2048], [32 / 63, 16 / 63, 8 / 63, 4 / 63, 2 / 63, 1 / 63], 256),
                          ([2, 8, 300], None, 256), ([2, 600], [0.5, 0.5], 512))
    ]
    tables["topousm_radii_norm"] = [
        [mr, mw, px, [None if x is None else list(x) for x in tile_compute._normalize_topousm_fast_radii_and_weights(
            None, None, px, manual_radii=mr, manual_weights=mw)]]
        for mr, mw, px in (([1], [1.0], 10.0), ([2.4, 8, 8.6, 0.2], None, 10.0), ([2, 8], [3, 1], 5.0),
                           ([2, "x", 8], [1, 1, 1], 1.0))
    ]
    np.savez_compressed(os.path.join(HERE, "encoding.npz"), **arrays)
    with open(os.path.join(HERE, "tables.json"), "w") as f:
        json.dump(tables, f, indent=1, sort_keys=True, default=float)
    print("golden fixtures written to", HERE)


AO_SPATIAL_RADII = (8.0, 40.0, 100.0)   # decimation factors 1, 2, 4 at 5 m (algorithm factor 1.5)


def main_ambient_occlusion():
    """ambient_occlusion.npz / .json: compute_ambient_occlusion_block and its spatial block."""
    ref = reference_shim.load()
    _stub_rasterio()
    import importlib
    ao_mod = ref._impl_ambient_occlusion
    db = importlib.import_module("FujiShaderGPU.algorithms.tile.dask_bridge")
    arrays = {}
    meta = {}
    a1 = _with_disks(synth.fbm(72, 90, hurst=0.7, seed=41, lo=0.0, hi=900.0), 4, 42, 2.0, 7.0)
    yy, xx = np.mgrid[0:61, 0:61]
    peak = (300.0 - 12.0 * np.sqrt((xx - 30.0) ** 2 + (yy - 30.0) ** 2)).astype(np.float32)
    a5 = synth.fbm(40, 50, hurst=0.8, seed=43, lo=0.0, hi=400.0)
    a5[10:13, 20:24] = np.nan
    cases = [
        # name, dem, num_samples, radius, intensity, pixel_size, psx, psy
        ("a1_fbm_nan", a1, 16, 10.0, 1.0, 5.0, 5.0, -5.0),
        ("a2_aniso", a1[:50, :64].copy(), 8, 5.5, 0.7, 4.0, 3.0, -5.0),
        ("a3_r1", a1[:30, :41].copy(), 12, 1.0, 1.0, 2.0, None, None),
        ("a4_peak_pit", np.concatenate([peak, -peak], axis=1), 16, 6.0, 2.0, 1.0, None, None),
        ("a5_wide_radius", a5, 16, 30.0, 1.0, 2.0, 2.0, -2.0),
        ("a6_flat", np.full((20, 24), 7.0, np.float32), 16, 4.0, 1.0, 1.0, None, None),
    ]
    for n, d, ns, r, it, px, psx, psy in cases:
        arrays[f"{n}/dem"] = d
        arrays[f"{n}/ao"] = ao_mod.compute_ambient_occlusion_block(
            d.copy(), num_samples=ns, radius=r, intensity=it, pixel_size=px,
            pixel_scale_x=psx, pixel_scale_y=psy)
        meta[n] = {"num_samples": ns, "radius": r, "intensity": it, "pixel_size": px, "psx": psx, "psy": psy}
    # the tile path's direct call with the display stretch (algorithms/tile/dask_bridge.py:190-203)
    arrays["a1_fbm_nan/direct_stretch"] = db._direct_ambient_occlusion(
        a1.copy(), dict(num_samples=16, radius=10.0, intensity=1.0, pixel_size=5.0, pixel_scale_x=5.0,
                        pixel_scale_y=-5.0, global_stats=(0.55, 0.4)))
    sp = synth.fbm(120, 136, hurst=0.8, seed=44, lo=0.0, hi=2500.0)
    sp_nan = _with_disks(sp, 4, 45, 6.0, 14.0)
    for dn, d in (("clean", sp), ("nan", sp_nan)):
        arrays[f"spatial_{dn}/dem"] = d
        for r in AO_SPATIAL_RADII:
            arrays[f"spatial_{dn}/ao_{int(r)}"] = ao_mod.compute_ambient_occlusion_spatial_block(
                d.copy(), num_samples=16, radius=r, intensity=1.0, pixel_size=5.0,
                pixel_scale_x=5.0, pixel_scale_y=-5.0)
    np.savez_compressed(os.path.join(HERE, "ambient_occlusion.npz"), **arrays)
    with open(os.path.join(HERE, "ambient_occlusion.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


def _stub_gdal_modules():
    """dem_preprocess imports rasterio and osgeo.gdal at module level; the functions the
    fixtures call use neither, so empty stand-ins let the module import."""
    import types
    for name in ("rasterio", "rasterio.enums", "rasterio.windows", "osgeo", "osgeo.gdal"):
        if name not in sys.modules:
            sys.modules[name] = types.ModuleType(name)
    sys.modules["rasterio.enums"].Resampling = type("Resampling", (), {"nearest": 0, "average": 5})
    sys.modules["rasterio.windows"].Window = object
    sys.modules["rasterio.windows"].transform = lambda *a, **k: None
    sys.modules["osgeo"].gdal = sys.modules["osgeo.gdal"]


def main_prepare():
    """prepare.npz / .json: push-pull fill, the NaN-aware coarse average, the NoData detection
    rules, the edge-connected mask and the per-band normalise-and-fill
    (io/dem_preprocess.py, algorithms/_pyramid_fill.py, utils/nodata_handler.py)."""
    reference_shim.load()
    _stub_gdal_modules()
    import importlib
    from scipy.ndimage import zoom as sp_zoom
    pf = importlib.import_module("FujiShaderGPU.algorithms._pyramid_fill")
    nh = importlib.import_module("FujiShaderGPU.utils.nodata_handler")
    dp = importlib.import_module("FujiShaderGPU.io.dem_preprocess")
    arrays, meta = {}, {}
    rng = np.random.default_rng(61)
    # push-pull fill
    c1 = synth.fbm(40, 56, hurst=0.8, seed=62, lo=0.0, hi=1200.0)
    v1 = ~synth.nodata_disks(40, 56, count=4, seed=63, rmin=2.0, rmax=7.0)
    v1[:, :5] = False
    c2 = synth.fbm(3, 70, hurst=0.8, seed=64, lo=0.0, hi=500.0)
    v2 = np.ones((3, 70), bool)
    v2[:, 20:62] = False
    c3 = synth.fbm(17, 9, hurst=0.8, seed=65, lo=0.0, hi=50.0)
    v3 = rng.random((17, 9)) > 0.7
    for n, c, v in (("pp1", c1, v1), ("pp2_wide", c2, v2), ("pp3_sparse", c3, v3),
                    ("pp4_all_valid", c3, np.ones_like(v3)), ("pp5_none_valid", c3, np.zeros_like(v3))):
        arrays[f"{n}/coarse"], arrays[f"{n}/valid"] = c, v
        arrays[f"{n}/filled"] = pf.pushpull_fill(c.copy(), v.copy(), xp=np, zoom=sp_zoom)
    # NaN-aware coarse average of a k x k oversampled nearest sample
    sm = synth.fbm(48, 64, hurst=0.7, seed=66, lo=-20.0, hi=800.0)
    sm[:, :10] = -9999.0
    sm[30:34, 40:44] = 0.0
    sm[5:9, 50:60] = np.nan
    decl = np.zeros(sm.shape, bool)
    decl[20:24, 20:28] = True
    arrays["avg/sample"], arrays["avg/declared"] = sm, decl
    co, cm = dp._nan_aware_coarse_average(None, 12, 16, None, [-9999.0, 0.0], oversample=4,
                                          sample_ma=np.ma.masked_array(sm, mask=decl))
    arrays["avg/coarse"], arrays["avg/void"] = co, cm
    # NoData detection rules
    det = {}
    frame = synth.fbm(64, 64, hurst=0.7, seed=67, lo=10.0, hi=900.0)
    frame[:6, :] = 0.0
    frame[-6:, :] = 0.0
    frame[:, :6] = 0.0
    frame[:, -6:] = 0.0
    spread = synth.fbm(64, 64, hurst=0.7, seed=68, lo=10.0, hi=900.0)
    spread[rng.random((64, 64)) < 0.1] = -9999.0
    extreme = synth.fbm(64, 64, hurst=0.7, seed=69, lo=10.0, hi=900.0)
    extreme[rng.random((64, 64)) < 0.08] = 10.0
    midval = synth.fbm(64, 64, hurst=0.7, seed=70, lo=10.0, hi=900.0)
    midval[rng.random((64, 64)) < 0.08] = 500.0
    for n, a in (("frame", frame), ("spread", spread), ("extreme", extreme), ("midval", midval),
                 ("clean", synth.fbm(64, 64, hurst=0.7, seed=71, lo=10.0, hi=900.0))):
        valid = np.isfinite(a)
        arrays[f"det_{n}/sample"] = a
        det[n] = [dp._detect_sentinel_nodata(a, valid, min_fraction=0.05),
                  dp._detect_border_nodata(a, valid, min_border_fraction=0.5)]
    meta["detect"] = det
    meta["coarse_shape"] = [[w, h, m, list(dp._coarse_shape(w, h, m))]
                            for w, h, m in ((65536, 32768, 2048), (1000, 3000, 2048), (100, 50, 2048),
                                            (5000, 5000, 2048), (4097, 2049, 1024))]
    # edge-connected mask
    em = rng.random((50, 60)) < 0.45
    arrays["edge/mask"] = em
    arrays["edge/connected"] = nh._edge_connected_mask(em)
    # per-band normalise-and-fill (enclosed and all), band at a row offset
    H, W = 96, 120
    full = synth.fbm(H, W, hurst=0.8, seed=72, lo=0.0, hi=1500.0)
    holes = synth.nodata_disks(H, W, count=4, seed=73, rmin=3.0, rmax=9.0)
    full[holes] = -9999.0
    full[:, :8] = np.nan
    ch, cw = 24, 30   # the full band itself as the 4x oversampled sample
    cavg, cvoid = dp._nan_aware_coarse_average(None, ch, cw, None, [-9999.0], oversample=4,
                                               sample_ma=np.ma.masked_array(full, mask=np.zeros((H, W), bool)))
    cvalid = (~cvoid) & np.isfinite(cavg)
    surface = pf.pushpull_fill(cavg, cvalid, xp=np, zoom=sp_zoom)
    ext = nh._edge_connected_mask(~cvalid)
    arrays["band/full"], arrays["band/surface"], arrays["band/exterior"] = full, surface, ext
    arrays["band/coarse"], arrays["band/cvalid"] = cavg, cvalid
    row_off, bh = 40, 33
    band = np.ma.masked_array(full[row_off:row_off + bh], mask=np.zeros((bh, W), bool))
    for mode, out_nd in (("enclosed", float("nan")), ("all", None)):
        arrays[f"band/{mode}"] = dp._apply_band_fill(
            band, row_off=row_off, bh=bh, width=W, height=H, ch=ch, cw=cw, do_fill=True, surface=surface,
            exterior_coarse=ext if mode == "enclosed" else None, extra_nodata=[-9999.0], fill_mode=mode,
            out_nodata=out_nd)
    fv, ex = dp._sample_coarse(surface, ext, row_off, bh, W, H, ch, cw)
    arrays["band/sample_vals"], arrays["band/sample_ext"] = fv, ex
    meta["band"] = {"row_off": row_off, "bh": bh, "ch": ch, "cw": cw}
    np.savez_compressed(os.path.join(HERE, "prepare.npz"), **arrays)
    with open(os.path.join(HERE, "prepare.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


SECTIONS = {"ambient_occlusion": lambda: main_ambient_occlusion(), "prepare": lambda: main_prepare()}


if __name__ == "__main__":
    if "--reference" in sys.argv:
        os.environ["FSG_REFERENCE_ROOT"] = sys.argv[sys.argv.index("--reference") + 1]
    # "--section <name>" regenerates that fixture alone
    if "--section" in sys.argv:
        SECTIONS[sys.argv[sys.argv.index("--section") + 1]]()
    else:
        main()
        for fn in SECTIONS.values():
            fn()
