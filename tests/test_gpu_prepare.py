"""GPU parity of the prepare step (NoData detection and void fill,
io/dem_preprocess.py / algorithms/_pyramid_fill.py of the reference) against the
reference's golden outputs and the CPU oracle.  Every piece is integer / float32
arithmetic in the reference's order with scipy's float64 interpolation, so the
bar is bit-exact."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from oracle import restated as R

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300 import _native as N
    return N


def _golden(golden_dir):
    g = np.load(os.path.join(golden_dir, "prepare.npz"))
    with open(os.path.join(golden_dir, "prepare.json")) as f:
        m = json.load(f)
    return g, m


def _eq(got, ref, what):
    got = got.cpu().numpy() if hasattr(got, "cpu") else np.asarray(got)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    assert np.array_equal(got, ref, equal_nan=True), \
        f"{what}: {int((~((got == ref) | (np.isnan(got) & np.isnan(ref)))).sum())} cells differ"


def _s():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("case", ["pp1", "pp2_wide", "pp3_sparse", "pp4_all_valid", "pp5_none_valid"])
def test_pushpull_matches_reference_golden(lib, golden_dir, case):
    g, _ = _golden(golden_dir)
    c = torch.from_numpy(g[f"{case}/coarse"]).cuda()
    v = torch.from_numpy(g[f"{case}/valid"].astype(np.uint8)).cuda()
    h, w = c.shape
    out = torch.full((h, w), -1.0, device="cuda")
    lib.check(lib.lib().fsg_pushpull_fill(_p(c), w, _p(v), w, h, w, _p(out), w, _s()))
    _eq(out, g[f"{case}/filled"], case)


def test_coarse_average_and_edge_mask_match_reference_golden(lib, golden_dir):
    g, _ = _golden(golden_dir)
    sm = torch.from_numpy(g["avg/sample"]).cuda()
    decl = torch.from_numpy(g["avg/declared"].astype(np.uint8)).cuda()
    coarse = torch.empty((12, 16), device="cuda")
    valid = torch.empty((12, 16), device="cuda", dtype=torch.uint8)
    vals = (C.c_double * 2)(-9999.0, 0.0)
    anyv = C.c_int32(0)
    lib.check(lib.lib().fsg_coarse_average(_p(sm), 64, _p(decl), 64, 12, 16, 4, vals, 2, _p(coarse), 16, _p(valid),
                                           16, C.byref(anyv), _s()))
    _eq(coarse, g["avg/coarse"], "coarse")
    assert np.array_equal(valid.cpu().numpy() == 0, g["avg/void"])
    assert anyv.value == int(g["avg/void"].any())
    m = torch.from_numpy(g["edge/mask"].astype(np.uint8)).cuda()
    h, w = m.shape
    out = torch.empty((h, w), device="cuda", dtype=torch.uint8)
    lib.check(lib.lib().fsg_edge_connected(_p(m), w, h, w, 0, _p(out), w, _s()))
    assert np.array_equal(out.cpu().numpy().astype(bool), g["edge/connected"])
    inv = (1 - m).contiguous()
    lib.check(lib.lib().fsg_edge_connected(_p(inv), w, h, w, 1, _p(out), w, _s()))
    assert np.array_equal(out.cpu().numpy().astype(bool), g["edge/connected"])


def test_edge_mask_spiral_needs_many_passes(lib):
    """A 1-pixel spiral corridor from the border to the centre crosses many 32 x 32
    tiles; the propagation relaunches until it settles."""
    n = 200
    m = np.zeros((n, n), bool)
    y0, x0, y1, x1 = 0, 0, n - 1, n - 1
    while y0 <= y1 and x0 <= x1:
        m[y0, x0:x1 + 1] = True
        m[y0:y1 + 1, x1] = True
        m[y1, x0:x1 + 1] = True
        m[y0 + 2:y1 + 1, x0] = True
        if y0 + 2 <= y1:
            m[y0 + 2, x0:x1 - 1] = True
        y0, x0, y1, x1 = y0 + 2, x0 + 2, y1 - 2, x1 - 2
    m[n // 2 + 5:n // 2 + 9, n // 2 - 3] = True   # a pocket
    ref = R.edge_connected_mask(m)
    mt = torch.from_numpy(m.astype(np.uint8)).cuda()
    out = torch.empty((n, n), device="cuda", dtype=torch.uint8)
    lib.check(lib.lib().fsg_edge_connected(_p(mt), n, n, n, 0, _p(out), n, _s()))
    assert np.array_equal(out.cpu().numpy().astype(bool), ref)


def test_band_fill_matches_reference_golden(lib, golden_dir):
    g, m = _golden(golden_dir)
    b = m["band"]
    full = torch.from_numpy(g["band/full"]).cuda()
    H, W = full.shape
    surf = torch.from_numpy(g["band/surface"]).cuda()
    ext = torch.from_numpy(g["band/exterior"].astype(np.uint8)).cuda()
    ch, cw = b["ch"], b["cw"]
    vals = (C.c_double * 1)(-9999.0)
    for mode, code in (("enclosed", 1), ("all", 2)):
        out = torch.empty((b["bh"], W), device="cuda")
        nf = C.c_int32(-1)
        lib.check(lib.lib().fsg_fill_apply(_p(full), W, H, W, b["row_off"], b["bh"], float("nan"), 0, vals, 1, code,
                                           _p(surf), cw, _p(ext), cw, ch, cw, _p(out), W, C.byref(nf), _s()))
        _eq(out, g[f"band/{mode}"], mode)
        assert nf.value == 0


@pytest.mark.parametrize("fill_mode", ["enclosed", "all", "none"])
def test_prepare_pipeline_matches_oracle(lib, fill_mode):
    """Declared NoData (-32768), an undeclared exterior frame of 0 (detected by the
    border rule), interior NaN voids; coarse grid 96 x 128 (oversample 4)."""
    from fujishadergpu_gb300 import synth
    from fujishadergpu_gb300.io import dem_preprocess as P
    H, W = 480, 640
    dem = synth.fbm(H, W, hurst=0.8, seed=201, lo=50.0, hi=2500.0)
    dem[synth.nodata_disks(H, W, count=8, seed=202, rmin=4.0, rmax=25.0)] = np.nan
    dem[:40, :] = 0.0
    dem[:, -50:] = 0.0
    dem[300:310, 100:140] = -32768.0
    res = P.prepare_dem(torch.from_numpy(dem).cuda(), nodata=-32768.0, fill_mode=fill_mode, coarse_max=128)
    ref, info = R.prepare_dem(dem, nodata=-32768.0, fill_mode=fill_mode, coarse_max=128)
    assert res.extra_nodata == info["extra_nodata"] == [0.0]
    assert res.coarse_shape == info["coarse_shape"] and res.oversample == info["oversample"]
    assert res.do_fill == info["do_fill"]
    _eq(res.array, ref, fill_mode)
    if fill_mode == "all":
        assert np.isfinite(res.array.cpu().numpy()).all()


def test_prepare_without_nodata_is_identity_and_override(lib):
    from fujishadergpu_gb300 import synth
    from fujishadergpu_gb300.io import dem_preprocess as P
    dem = synth.fbm(200, 260, hurst=0.8, seed=203, lo=50.0, hi=900.0)
    res = P.prepare_dem(torch.from_numpy(dem).cuda(), coarse_max=64)
    assert not res.do_fill and res.extra_nodata == []
    _eq(res.array, dem, "identity")
    # an explicit override sentinel spread inside the raster (enclosed voids filled)
    dem2 = dem.copy()
    dem2[80:90, 100:130] = -1.0
    res = P.prepare_dem(torch.from_numpy(dem2).cuda(), coarse_max=64, nodata_override=-1.0)
    ref, info = R.prepare_dem(dem2, coarse_max=64, nodata_override=-1.0)
    assert res.extra_nodata == info["extra_nodata"]
    _eq(res.array, ref, "override")
    with pytest.raises(ValueError):
        P.prepare_dem(torch.from_numpy(dem).cuda(), fill_mode="bogus")


def test_value_statistics_match_numpy_unique(lib, golden_dir):
    """fsg_value_mode against np.unique + argmax (the detection rule's statistics): the
    golden detection samples, ties (the smaller value wins), -0 and +0 as one value, and
    declared cells left out."""
    g, _ = _golden(golden_dir)
    rng = np.random.default_rng(5)
    tie = rng.integers(-3, 4, size=(300, 257)).astype(np.float32)
    tie[tie == 0] = np.float32(-0.0)
    tie[::7, ::3] = 0.0
    tie[5:9, :] = np.nan
    decl = np.zeros(tie.shape, bool)
    decl[100:140, 17:90] = True
    samples = [(g[f"det_{n}/sample"], None) for n in ("frame", "spread", "extreme", "midval", "clean")]
    samples += [(tie, decl), (tie, None)]
    for a, d in samples:
        t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
        h, w = a.shape
        dm = torch.from_numpy((d if d is not None else np.zeros(a.shape, bool)).astype(np.uint8)).cuda()
        nf, lo, hi, mv, mc = C.c_int64(), C.c_double(), C.c_double(), C.c_double(), C.c_int64()
        lib.check(lib.lib().fsg_value_mode(_p(t), w, h, w, _p(dm), w, 0.05, C.byref(nf), C.byref(lo), C.byref(hi),
                                           C.byref(mv), C.byref(mc), _s()))
        valid = np.isfinite(a) & ~(d if d is not None else np.zeros(a.shape, bool))
        fin = a[valid]
        vals, counts = np.unique(fin, return_counts=True)
        assert nf.value == fin.size
        assert lo.value == float(vals[0]) and hi.value == float(vals[-1])
        i = int(np.argmax(counts))
        if counts[i] / float(fin.size) >= 0.05:
            assert mc.value == int(counts[i]) and mv.value == float(vals[i])
        else:
            assert mc.value == 0 or mc.value / float(fin.size) < 0.05
        c = C.c_int64()
        lib.check(lib.lib().fsg_count_equal(_p(t), w, h, w, float(vals[i]), C.byref(c), _s()))
        assert c.value == int(np.sum(a == np.float32(vals[i])))
