"""Host-side checks of polynomial constants compiled into the kernels: the coefficients are
read from the CUDA source and evaluated in float32 the way the kernel does (Horner on t^2
with fused multiply-adds, emulated in float64 and rounded once per step), so an edit that
breaks the stated error bound or the reference's cap fails here without a GPU."""
import os
import re

import numpy as np

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "fujishadergpu_gb300", "csrc")


def _occlusion_coefficients():
    src = open(os.path.join(CSRC, "fsg_ao.cu")).read()
    body = src[src.index("occlusion2("):]
    body = body[: body.index("return __fmul2_rn(t, p);")]
    k = re.search(r"constexpr double OCC_K = ([0-9.eE+-]+) \* \(1\.0 - 1\.0 / ([0-9.]+)\);", src)
    scale = float(k.group(1)) * (1.0 - 1.0 / float(k.group(2)))
    # highest coefficient first, as the Horner steps appear in the source
    hexes = re.findall(r"\(float\)\((-?0x[0-9a-fA-F.]+p-?\d+) \* OCC_K\)", body)
    return [np.float32(float.fromhex(h) * scale) for h in hexes]


def test_occlusion_polynomial_error_and_cap():
    """min(atan(t) / (pi/4), 1) for t in [0, 1] within 1e-6 (normalised occlusion units), and a
    saturated ratio (t = 1) gives at most 1, the reference's cap."""
    coef = _occlusion_coefficients()
    assert len(coef) >= 5
    t = np.linspace(0.0, 1.0, 200001, dtype=np.float32)
    t2 = (t * t).astype(np.float32)
    p = np.full_like(t2, coef[0])
    for c in coef[1:]:
        p = (t2.astype(np.float64) * p.astype(np.float64) + np.float64(c)).astype(np.float32)
    occ = (t * p).astype(np.float32)
    ref = np.minimum(np.arctan(t.astype(np.float64)) / (np.pi / 4.0), 1.0)
    assert np.max(np.abs(occ.astype(np.float64) - ref)) <= 1e-6
    assert occ[-1] <= 1.0 and occ.max() <= 1.0


def _horner_coefficients(path, start, end, pattern):
    src = open(os.path.join(CSRC, path)).read()
    body = src[src.index(start):]
    body = body[: body.index(end)]
    return [np.float32(float.fromhex(h)) for h in re.findall(pattern, body)]


def _odd_poly32(coef, a):
    a2 = (a * a).astype(np.float32)
    p = np.full_like(a2, coef[0])
    for c in coef[1:]:
        p = (a2.astype(np.float64) * p.astype(np.float64) + np.float64(c)).astype(np.float32)
    return (a * p).astype(np.float32)


def test_atan_poly_error():
    """atan_poly (fsg_common.cuh): |atan(a) - a P(a^2)| <= 1.5e-7 rad on [0, 1]."""
    coef = _horner_coefficients("fsg_common.cuh", "float atan_poly(float x)", "float r = a * p;",
                                r"(-?0x[0-9a-fA-F.]+p[-+]?\d+)f")
    assert len(coef) == 8
    a = np.linspace(0.0, 1.0, 200001, dtype=np.float32)
    err = np.abs(_odd_poly32(coef, a).astype(np.float64) - np.arctan(a.astype(np.float64)))
    assert err.max() <= 1.5e-7


def test_slope_degree_polynomial_error():
    """atan_deg_pos2 (fsg_stencil.cu): |degrees(atan(a)) - a P(a^2)| <= 1.1e-4 degree on [0, 1]."""
    coef = _horner_coefficients("fsg_stencil.cu", "f2 atan_deg_pos2(f2 x)", "f2 r = mul2(a, p);",
                                r"S2\((-?0x[0-9a-fA-F.]+p[-+]?\d+)f\)")
    assert len(coef) == 6
    a = np.linspace(0.0, 1.0, 200001, dtype=np.float32)
    err = np.abs(_odd_poly32(coef, a).astype(np.float64) - np.degrees(np.arctan(a.astype(np.float64))))
    assert err.max() <= 1.1e-4
