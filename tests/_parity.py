"""Comparison helpers shared by the GPU parity tests.

Tolerances (stated once, used everywhere):
  * NaN / NoData masks: identical.
  * float32 stencil and topousm outputs: |gpu - ref| <= 1e-5 x (output range).
  * int16 / uint8 codes: within 1 LSB.
  * curvature display ((tanh(100k)+1)/2)^(1/2.2): 1e-5, or, where tanh(100k)
    is within a few float32 ulps of -1 (the gamma step amplifies the last bit
    of tanh there; NumPy's and CUDA's float32 tanh differ in that bit), the
    pre-gamma value (tanh+1)/2 agrees to 4 ulps of tanh (2^-23); and, at cells
    where the reference's own float32 curvature is ill-conditioned (its
    numerator's terms cancel), 1e-5 plus twice the distance between the
    reference's float32 and float64 results there.
  * exact openness: mean angle within 0.01 degree.
  * ambient occlusion (output in [0, 1]): 1e-5 (a polynomial for the normalised
    occlusion atan(t) / (pi/4), within 6.3e-7, and a reciprocal multiply stand in
    for float32 atan and division).
  * a weighted combination of curvature displays (spatial mode): 1e-5 plus
    the sum over responses of weight x that response's own allowance (1e-5,
    or in its tail the display change of 2^-23 in the pre-gamma value).
"""
from __future__ import annotations

import numpy as np

CURV_TAIL_TOL = 2.0 ** -23


def to_np(x):
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def assert_same_nan(got, ref, what=""):
    gn, rn = np.isnan(got), np.isnan(ref)
    bad = np.argwhere(gn != rn)
    assert bad.size == 0, f"{what}: NaN mask differs at {bad[:5].tolist()} ({len(bad)} cells)"


def assert_close_range(got, ref, rng, what="", rel=1e-5):
    got = to_np(got)
    ref = to_np(ref)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    assert_same_nan(got, ref, what)
    m = ~np.isnan(ref)
    if not m.any():
        return 0.0
    d = np.abs(got[m].astype(np.float64) - ref[m].astype(np.float64))
    tol = rel * rng
    worst = float(d.max())
    assert worst <= tol, f"{what}: max |diff| {worst:.3e} > {tol:.3e} at {np.argmax(d)}"
    return worst


def assert_close_rel(got, ref, what="", rel=1e-5, atol=0.0):
    got = to_np(got)
    ref = to_np(ref)
    assert_same_nan(got, ref, what)
    m = ~np.isnan(ref)
    d = np.abs(got[m].astype(np.float64) - ref[m].astype(np.float64))
    lim = rel * np.abs(ref[m].astype(np.float64)) + atol
    bad = d > lim
    assert not bad.any(), f"{what}: {int(bad.sum())} cells over rel {rel}; worst {float((d - lim).max()):.3e}"


def assert_curvature_close(got, ref, what="", ref64_at=None):
    """Display-domain 1e-5, or the pre-gamma tail rule described in the module docstring.

    ``ref64_at(ys, xs)`` (optional) gives the same algorithm in float64 at those cells:
    where the reference's own float32 result is ill-conditioned (its numerator's terms
    cancel), a cell also passes when |got - ref| <= 1e-5 + 2 |ref - ref64|, i.e. within
    twice the reference's own float32 error there."""
    got = to_np(got).astype(np.float64)
    ref = to_np(ref).astype(np.float64)
    assert_same_nan(got, ref, what)
    m = ~np.isnan(ref)
    g, r = got[m], ref[m]
    d = np.abs(g - r)
    ok = d <= 1e-5
    ug, ur = g ** 2.2, r ** 2.2
    tail = (~ok) & (np.minimum(ug, ur) < 1e-4) & (np.abs(ug - ur) <= CURV_TAIL_TOL)
    bad = ~(ok | tail)
    if bad.any() and ref64_at is not None:
        ys, xs = np.nonzero(m)
        ys, xs = ys[bad], xs[bad]
        r64 = np.asarray(ref64_at(ys, xs), dtype=np.float64)
        own = np.abs(r[bad] - r64)
        cond = d[bad] <= 1e-5 + 2.0 * own
        idx = np.flatnonzero(bad)
        bad[idx[cond]] = False
    assert not bad.any(), (f"{what}: {int(bad.sum())} cells off; worst display diff "
                           f"{float(d[bad].max()):.3e}")
    return int(tail.sum())


def curvature_allowance(ref):
    """Per-cell display allowance of one curvature response (the rule of assert_curvature_close)."""
    r = to_np(ref).astype(np.float64)
    u = r ** 2.2
    tail = np.abs((u + CURV_TAIL_TOL) ** (1 / 2.2) - r)
    return np.where(u < 1e-4, np.maximum(tail, 1e-5), 1e-5)


def assert_curvature_combined_close(got, ref, responses, weights, what=""):
    """A weighted sum of curvature displays against the oracle's, each response allowed its own error."""
    got = to_np(got).astype(np.float64)
    ref = to_np(ref).astype(np.float64)
    assert_same_nan(got, ref, what)
    allow = np.full(ref.shape, 1e-5)
    for resp, w in zip(responses, weights):
        allow = allow + float(w) * np.nan_to_num(curvature_allowance(resp), nan=0.0)
    m = ~np.isnan(ref)
    d = np.abs(got - ref)
    bad = m & (d > allow)
    assert not bad.any(), (f"{what}: {int(bad.sum())} cells off; worst excess "
                           f"{float((d - allow)[bad].max()):.3e}")


def assert_codes_close(got, ref, what="", lsb=1):
    got = to_np(got).astype(np.int64)
    ref = to_np(ref).astype(np.int64)
    d = np.abs(got - ref)
    assert int(d.max(initial=0)) <= lsb, f"{what}: max code diff {int(d.max())}"
    # NoData code 0 exactly where the reference has it
    assert np.array_equal(got == 0, ref == 0) or lsb > 0
