"""The tensor-core path of topousm_fast (fsg_topousm_tc.cu: split-BF16 banded
Toeplitz products of the full-resolution box means on tcgen05, FP32
accumulation; tiles holding NoData recomputed by the exact kernel).

Tolerance: the error against the same algorithm in float64 (the oracle with
dtype float64) is at most 1e-5 of p99(|result|), the normalisation scale of
topousm_fast (_normalization.py:21-41), i.e. 1e-5 in normalised output units.
NaN masks are identical.  Against the exact CUDA-core path the same bound
applies twice over (both are within it of the float64 result).
"""
import numpy as np
import pytest

from oracle import restated as R
from tests._parity import assert_codes_close, assert_same_nan, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

W6 = [w / 63.0 for w in (32, 16, 8, 4)]


@pytest.fixture(scope="module")
def tu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300 import _native as N
    from fujishadergpu_gb300.algorithms import _impl_topousm_fast
    N.kernel_errors()  # start from a clear error word
    return _impl_topousm_fast


def _dem(h, w, seed, disks=0):
    from fujishadergpu_gb300 import synth
    d = synth.fbm_ridged(h, w, hurst=0.8, seed_fbm=seed, seed_ridged=seed + 1, lo=0.0, hi=3500.0)
    if disks:
        d[synth.nodata_disks(h, w, count=disks, seed=seed + 2, rmin=4.0, rmax=20.0)] = np.nan
    return d


def _rel_err(got, ref64):
    scale = R.topousm_scale(ref64)[0]
    assert_same_nan(got, ref64, "tensor path")
    m = ~np.isnan(ref64)
    return float(np.abs(got.astype(np.float64)[m] - ref64[m]).max()) / scale


@pytest.mark.parametrize("shape,radii,weights", [
    ((700, 910), [2, 8, 32, 128], W6),
    ((300, 340), [2, 8, 32], [0.5, 0.3, 0.2]),
    ((129, 193), [3, 17], [0.6, 0.4]),          # one CTA tile plus one row / column
    ((90, 75), [2, 8, 32], [0.5, 0.3, 0.2]),    # window smaller than a CTA tile and than 2R+1
    ((520, 640), [5], [1.0]),                   # a single full-resolution radius
])
def test_tensor_path_vs_fp64_oracle_without_nodata(tu, shape, radii, weights):
    from fujishadergpu_gb300 import _native as N
    dem = _dem(*shape, seed=81)
    d = torch.from_numpy(dem).cuda()
    got = to_np(tu.compute_topousm_fast_efficient_block(d, radii=radii, weights=weights, pixel_size=10.0,
                                                         path="tensor"))
    exact = to_np(tu.compute_topousm_fast_efficient_block(d, radii=radii, weights=weights, pixel_size=10.0))
    ref64 = R.topousm_block(dem.astype(np.float64), radii=radii, weights=weights, pixel_size=10.0)
    e_t, e_x = _rel_err(got, ref64), _rel_err(exact, ref64)
    assert e_t <= 1e-5, (e_t, e_x)
    assert e_x <= 1e-5, e_x
    assert not np.array_equal(got, exact), "the tensor path did not run (identical to the exact path)"
    assert N.kernel_errors() == 0


def test_tiles_with_nodata_take_the_exact_kernel(tu):
    """A window with NoData disks: tiles whose 192 x 256 input region holds NoData are
    recomputed by the exact kernel (bit-identical to the exact path there); the rest
    come from the tensor cores."""
    from fujishadergpu_gb300 import _native as N
    dem = _dem(640, 800, seed=91, disks=3)
    d = torch.from_numpy(dem).cuda()
    radii = [2, 8, 32, 128]
    got = to_np(tu.compute_topousm_fast_efficient_block(d, radii=radii, weights=W6, pixel_size=10.0, path="tensor"))
    exact = to_np(tu.compute_topousm_fast_efficient_block(d, radii=radii, weights=W6, pixel_size=10.0))
    ref64 = R.topousm_block(dem.astype(np.float64), radii=radii, weights=W6, pixel_size=10.0)
    assert _rel_err(got, ref64) <= 1e-5
    nan = np.isnan(dem)
    same = 0
    for y0 in range(0, 640, 128):
        for x0 in range(0, 800, 192):
            region = nan[max(0, y0 - 32):y0 + 160, max(0, x0 - 32):x0 + 224]
            tile_g, tile_x = got[y0:y0 + 128, x0:x0 + 192], exact[y0:y0 + 128, x0:x0 + 192]
            if region.any():
                assert np.array_equal(tile_g, tile_x, equal_nan=True), (y0, x0)
                same += 1
    assert same > 0, "no tile held NoData: the case does not exercise the fix-up"
    assert N.kernel_errors() == 0


@pytest.mark.parametrize("dtype", ["float32", "int16"])
def test_tile_loop_tensor_path_with_coarse_field(tu, dtype):
    """The tile loop (overview field for the large radii, global p99 scale, encoding)
    gives the same result through both paths."""
    from fujishadergpu_gb300.core import tile_loop
    dem = _dem(1100, 1300, seed=101, disks=2)
    d = torch.from_numpy(dem).cuda()
    kw = dict(tile_size=512, pixel_size=10.0, pixel_scale_x=10.0, pixel_scale_y=-10.0,
              radii=[2, 8, 32, 128, 512, 2048], weights=[w / 63.0 for w in (32, 16, 8, 4, 2, 1)],
              output_dtype=dtype)
    ex = tile_loop.process_dem_array(d, "topousm_fast", **kw)
    tc = tile_loop.process_dem_array(d, "topousm_fast", topousm_path="tensor", global_stats=ex.stats, **kw)
    a, b = to_np(tc.output), to_np(ex.output)
    if dtype == "float32":
        assert_same_nan(a, b, "tile loop")
        m = ~np.isnan(b)
        assert float(np.abs(a[m].astype(np.float64) - b[m]).max()) <= 2e-5
    else:
        assert_codes_close(a, b, "int16 codes")


def test_unsupported_radius_falls_back_to_the_exact_kernel(tu):
    dem = _dem(200, 260, seed=111)
    d = torch.from_numpy(dem).cuda()
    kw = dict(radii=[2, 40], weights=[0.5, 0.5], pixel_size=10.0)
    a = to_np(tu.compute_topousm_fast_efficient_block(d, path="tensor", **kw))
    b = to_np(tu.compute_topousm_fast_efficient_block(d, **kw))
    assert np.array_equal(a, b, equal_nan=True)


def test_unknown_path_is_rejected(tu):
    d = torch.zeros((16, 16), device="cuda")
    with pytest.raises(ValueError, match="unknown topousm path"):
        tu.compute_topousm_fast_efficient_block(d, radii=[2], weights=[1.0], path="fast")
