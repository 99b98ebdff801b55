"""Parity at the workload sizes the benchmark configurations name, not only on
small fixtures: the CUDA path is run over the whole raster (the product's own
tile grid, ``core.tile_loop``) and compared with the oracle on full tiles.

  * 2048^2 hillshade, one tile (plain float32 method).
  * 16384^2 fused hillshade + slope + profile / planform curvature, ~2-3 %
    NoData in seeded disks of radius 10-200 px, 4096^2 tiles with a 2 px halo,
    float32 and uint8 planes; the four corner tiles and the tile that the
    largest edge-crossing disk touches, each against the oracle on its
    clipped window.
  * topousm_fast on a 32768^2 fBm + ridged DEM, radii 2 ... 2048 (2^n weights),
    through the tile loop (large radii from the 2048^2 overview field, global
    p99 scale); sampled 4096^2 tiles against the same algorithm in float64.
  * exact openness, R = 256, 16 directions, positive and negative, reference
    and dense sampling, on a 1024^2 crop of a 16384^2 fBm + ridged DEM.

Host memory stays bounded: the comparison runs tile by tile.  Setting
``FSG_PARITY_REPORT`` to a file path writes the measured error figures there
as JSON lines.
"""
import json
import os

import numpy as np
import pytest

from oracle import restated as R
from tests._parity import assert_close_range, assert_codes_close, assert_curvature_close, assert_same_nan, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda")


def _report(**kw):
    path = os.environ.get("FSG_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(kw) + "\n")


def test_hillshade_2048_single_tile(cuda):
    from fujishadergpu_gb300 import algorithms as A
    from fujishadergpu_gb300 import synth
    dem = synth.fbm_device(2048, 2048, hurst=0.8, seed=1, lo=0.0, hi=3000.0)
    got = to_np(A.compute_hillshade_block(dem, azimuth=315, altitude=45, z_factor=1.0, pixel_size=10.0,
                                          pixel_scale_x=10.0, pixel_scale_y=-10.0))
    ref = R.hillshade(to_np(dem), pixel_size=10.0, psx=10.0, psy=-10.0)
    err = assert_close_range(got, ref, 1.0, "hillshade 2048^2")
    _report(case="hillshade_2048", max_abs_err=err)


STENCIL_OUT = {"hillshade": (0.0, 1.0), "slope": (0.0, 90.0), "curvature_profile": (0.0, 1.0),
               "curvature_planform": (0.0, 1.0)}


def _edge_disk_tile(h, w, tile, count, seed, rmin, rmax):
    """(ty, tx) of a tile touched by the largest disk that crosses a tile edge
    (the disks of synth.nodata_disks_device with the same seed)."""
    rng = np.random.default_rng(seed)
    cy, cx, rr = rng.uniform(0, h, count), rng.uniform(0, w, count), rng.uniform(rmin, rmax, count)
    best = None
    for y, x, r in zip(cy, cx, rr):
        crosses = (abs(x - round(x / tile) * tile) < r and 0 < round(x / tile) < w // tile) or \
                  (abs(y - round(y / tile) * tile) < r and 0 < round(y / tile) < h // tile)
        if crosses and (best is None or r > best[2]):
            best = (y, x, r)
    assert best is not None
    return int(best[0] // tile), int(best[1] // tile), float(best[2])


def test_fused_stencil_16384_tiles_float32_and_uint8(cuda):
    from fujishadergpu_gb300 import _arrays, synth
    from fujishadergpu_gb300.algorithms import _stencil as S
    from fujishadergpu_gb300.core import tile_loop
    from fujishadergpu_gb300.io.output_encoding import quantize_params
    H = W = 16384
    tile, halo = 4096, 2
    count, seed = 200, 12
    dem = synth.fbm_device(H, W, hurst=0.7, seed=2, lo=0.0, hi=4000.0)
    synth.nodata_disks_device(dem, count=count, seed=seed, rmin=10.0, rmax=200.0)
    frac = float(torch.isnan(dem).float().mean())
    infos = tile_loop.tile_grid(H, W, tile, halo)
    tiles = tile_loop.make_tiles(infos, pixel_scale_x=5.0, pixel_scale_y=-5.0)
    params = S.make_params(azimuth=315.0, altitude=45.0, pixel_size=5.0)
    view = _arrays.as_device_f32_2d(dem)
    f32 = {n: torch.empty((H, W), device=cuda) for n in STENCIL_OUT}
    u8 = {n: torch.empty((H, W), device=cuda, dtype=torch.uint8) for n in STENCIL_OUT}
    qps = {n: quantize_params(lo, hi, "uint8") for n, (lo, hi) in STENCIL_OUT.items()}
    S.launch(view, tiles, params, {S.OUTPUT_INDEX[n]: S.make_plane(t) for n, t in f32.items()})
    S.launch(view, tiles, params, {S.OUTPUT_INDEX[n]: S.make_plane(t, "uint8", qps[n]) for n, t in u8.items()})
    torch.cuda.synchronize()
    host = to_np(dem)
    ety, etx, er = _edge_disk_tile(H, W, tile, count, seed, 10.0, 200.0)
    picks = {(0, 0), (0, 3), (3, 0), (3, 3), (ety, etx)}
    oracle_grid = R.tile_grid(H, W, tile, halo)
    by_pos = {(t.ty, t.tx): t for t in infos}
    worst = {}
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in oracle_grid:
        if (ty, tx) not in picks:
            continue
        t = by_pos[(ty, tx)]
        assert (t.core_x, t.core_y, t.core_w, t.core_h, t.win_x, t.win_y, t.win_w, t.win_h) == \
            (cx, cy, cw, ch, wx, wy, ww, wh), "package tile grid differs from the reference's"
        win = host[wy:wy + wh, wx:wx + ww]
        core = (slice(cy - wy, cy - wy + ch), slice(cx - wx, cx - wx + cw))
        kw = dict(pixel_size=5.0, psx=5.0, psy=-5.0)
        refs = {"hillshade": R.hillshade(win, **kw), "slope": R.slope(win, **kw),
                "curvature_profile": R.curvature(win, curvature_type="profile", **kw),
                "curvature_planform": R.curvature(win, curvature_type="planform", **kw)}
        for n, ref in refs.items():
            ref = ref[core]
            g = to_np(f32[n][cy:cy + ch, cx:cx + cw])
            what = f"{n} tile {ty},{tx}"
            if n.startswith("curvature"):
                def ref64_at(ys, xs, ct=n.split("_")[1]):
                    out = []
                    for yy, xx in zip(ys + (cy - wy), xs + (cx - wx)):  # window coordinates
                        a0, b0 = max(0, yy - 12), max(0, xx - 12)
                        sub = win[a0:min(win.shape[0], yy + 13), b0:min(win.shape[1], xx + 13)]
                        # the sub-window's edges stay >= 12 px away unless they are the window's own
                        out.append(R.curvature(sub.astype(np.float64), curvature_type=ct, **kw)[yy - a0, xx - b0])
                    return out
                assert_curvature_close(g, ref, what, ref64_at=ref64_at)
                e = float(np.nanmax(np.abs(g.astype(np.float64) - ref)))
            else:
                e = assert_close_range(g, ref, STENCIL_OUT[n][1], what)
            worst[n] = max(worst.get(n, 0.0), e)
            assert_codes_close(to_np(u8[n][cy:cy + ch, cx:cx + cw]), R.quantize_array(ref, qps[n], "uint8"),
                               what + " uint8")
    _report(case="stencil_16384", nodata_frac=frac, tiles=sorted(picks), edge_disk_radius=er,
            max_abs_err=worst)


def test_topousm_32768_sampled_tiles_vs_fp64(cuda):
    from fujishadergpu_gb300 import synth
    from fujishadergpu_gb300.core import tile_loop
    H = W = 32768
    radii = [2, 8, 32, 128, 512, 2048]
    weights = [w / 63.0 for w in (32, 16, 8, 4, 2, 1)]
    dem = synth.fbm_ridged_device(H, W, hurst=0.8, seed_fbm=3, seed_ridged=4, lo=0.0, hi=3500.0)
    res = tile_loop.process_dem_array(dem, "topousm_fast", tile_size=4096, pixel_size=10.0, pixel_scale_x=10.0,
                                      pixel_scale_y=-10.0, radii=radii, weights=weights)
    scale = float(res.stats[0])
    pad = res.padding
    torch.cuda.synchronize()
    # FP64 overview of the whole raster (exact 16 x 16 block means) and the large-radius field
    dec = 16
    ov = np.empty((H // dec, W // dec), np.float64)
    for i in range(0, H, 1024):
        band = to_np(dem[i:i + 1024]).astype(np.float64)
        ov[i // dec:(i + 1024) // dec] = band.reshape(1024 // dec, dec, W // dec, dec).mean(axis=(1, 3))
    field64 = R.coarse_field(ov, large_radii=[512, 2048], large_weights=weights[4:], decimation=float(dec))
    small_r, small_w = radii[:4], weights[:4]
    out = res.output
    rep = []
    for (ty, tx) in ((0, 0), (3, 4), (7, 7)):
        cy, cx = ty * 4096, tx * 4096
        wy, wx = max(cy - pad, 0), max(cx - pad, 0)
        wy1, wx1 = min(cy + 4096 + pad, H), min(cx + 4096 + pad, W)
        win = to_np(dem[wy:wy1, wx:wx1]).astype(np.float64)
        small = R.topousm_block(win, radii=small_r, weights=small_w, pixel_size=10.0)
        # the field sampled at the reference's float32 pixel-centre coordinates, and in float64
        samp32 = R.bilinear_sample_coarse(field64.astype(np.float32), wy, wy1, wx, wx1, H, W, dtype=np.float32)
        coords = np.empty((2, wy1 - wy, wx1 - wx), np.float64)
        f = np.float32
        coords[0] = ((np.arange(wy, wy1, dtype=f) + f(0.5)) * f(field64.shape[0] / float(H)) - f(0.5))[:, None]
        coords[1] = ((np.arange(wx, wx1, dtype=f) + f(0.5)) * f(field64.shape[1] / float(W)) - f(0.5))[None, :]
        import scipy.ndimage as ndi
        samp_f32coords = ndi.map_coordinates(field64, coords, order=1, mode="nearest")
        samp64 = R.bilinear_sample_coarse(field64, wy, wy1, wx, wx1, H, W, dtype=np.float64)
        core = (slice(cy - wy, cy - wy + 4096), slice(cx - wx, cx - wx + 4096))
        w_large = sum(weights[4:])
        ref_a = ((small + w_large * win - samp_f32coords) / scale)[core]
        ref_b = ((small + w_large * win - samp64) / scale)[core]
        got = to_np(out[cy:cy + 4096, cx:cx + 4096]).astype(np.float64)
        assert_same_nan(got, ref_a, f"topousm tile {ty},{tx}")
        ea = float(np.nanmax(np.abs(got - ref_a)))
        eb = float(np.nanmax(np.abs(got - ref_b)))
        rng = float(np.nanmax(ref_b) - np.nanmin(ref_b))
        rep.append({"tile": [ty, tx], "max_abs_err_norm": ea, "max_abs_err_norm_fp64_coords": eb,
                    "rel_to_tile_range": ea / rng, "tile_range": rng, "samp32_vs_64": float(
                        np.nanmax(np.abs(samp32.astype(np.float64) - samp64)) / scale)})
        # normalised output (raw / p99|raw|): 1e-5 of p99|raw|, the same bound as the float32 parity gate
        assert ea <= 1e-5, (ty, tx, ea)
    _report(case="topousm_32768", scale=scale, padding=pad, tiles=rep)


@pytest.mark.parametrize("otype", ["positive", "negative"])
def test_openness_r256_crop_both_samplings(cuda, otype):
    from fujishadergpu_gb300 import algorithms as A
    from fujishadergpu_gb300 import synth
    big = synth.fbm_ridged_device(16384, 16384, hurst=0.7, seed_fbm=5, seed_ridged=6, lo=0.0, hi=3000.0)
    crop = big[8192:9216, 8192:9216].contiguous()
    del big
    host = to_np(crop)
    kw = dict(openness_type=otype, num_directions=16, max_distance=256, pixel_size=5.0)
    ref_kw = dict(kw, psx=5.0, psy=-5.0, raw_degrees=True)
    got = to_np(A.compute_openness_raw_degrees(crop, pixel_scale_x=5.0, pixel_scale_y=-5.0, **kw))
    ref = R.openness(host, **ref_kw)
    assert_same_nan(got, ref, "reference sampling")
    e_ref = float(np.nanmax(np.abs(got.astype(np.float64) - ref)))
    assert e_ref <= 0.01, e_ref
    dense = to_np(A.compute_openness_raw_degrees(crop, pixel_scale_x=5.0, pixel_scale_y=-5.0, sampling="dense",
                                                 **kw))
    offs = R.dense_offsets(16, 256)
    e_dense = 0.0
    for rows in ((0, 40), (500, 540)):
        r = R.openness(host, offsets=offs, rows=rows, **ref_kw)
        g = dense[rows[0]:rows[1]]
        assert_same_nan(g, r, f"dense rows {rows}")
        e_dense = max(e_dense, float(np.nanmax(np.abs(g.astype(np.float64) - r))))
    assert e_dense <= 0.01, e_dense
    _report(case=f"openness_r256_{otype}", max_abs_err_deg_reference=e_ref, max_abs_err_deg_dense=e_dense)
