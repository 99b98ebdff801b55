"""Seeded synthetic DEMs for tests and benchmarks.

The reference measures on no public dataset, so every workload here is
synthetic: spectral-synthesis fractional Brownian motion (fBm), ridged
multifractal value noise, NoData disks and geographic latitude bands.

Two implementations of the same recipe exist:

* ``numpy`` (``fbm``, ``ridged``, ``nodata_disks``) for small test rasters,
  bit-reproducible from ``numpy.random.default_rng(seed)``;
* ``torch`` (``fbm_device`` ...) for bench-sized rasters (up to 65536 x 32768),
  generated directly in device memory so a 4 GiB DEM does not have to be built
  on the host.  Same spectrum and rescaling, different random stream.
"""
from __future__ import annotations

import math
from typing import Optional, Tuple

import numpy as np


# --------------------------------------------------------------------------- numpy
def _rescale(a: np.ndarray, lo: float, hi: float) -> np.ndarray:
    amin = float(a.min())
    amax = float(a.max())
    span = amax - amin if amax > amin else 1.0
    return lo + (a - amin) * ((hi - lo) / span)


def fbm(h: int, w: int, *, hurst: float = 0.8, seed: int = 0,
        lo: float = 0.0, hi: float = 3000.0) -> np.ndarray:
    """2-D spectral-synthesis fBm: amplitude ~ |k|^-(H+1), random complex phases."""
    rng = np.random.default_rng(seed)
    ky = np.fft.fftfreq(h)[:, None]
    kx = np.fft.rfftfreq(w)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    amp = k ** (-(hurst + 1.0))
    amp[0, 0] = 0.0
    spec = amp * (rng.standard_normal(amp.shape) + 1j * rng.standard_normal(amp.shape))
    field = np.fft.irfft2(spec, s=(h, w))
    return _rescale(field, lo, hi).astype(np.float32)


def _value_noise(h: int, w: int, cell: float, rng: np.random.Generator) -> np.ndarray:
    gh = int(math.ceil(h / cell)) + 2
    gw = int(math.ceil(w / cell)) + 2
    lattice = rng.random((gh, gw)) * 2.0 - 1.0
    y = np.arange(h) / cell
    x = np.arange(w) / cell
    y0 = np.floor(y).astype(np.int64)
    x0 = np.floor(x).astype(np.int64)
    fy = y - y0
    fx = x - x0
    fy = fy * fy * (3.0 - 2.0 * fy)
    fx = fx * fx * (3.0 - 2.0 * fx)
    a = lattice[y0[:, None], x0[None, :]]
    b = lattice[y0[:, None], x0[None, :] + 1]
    c = lattice[y0[:, None] + 1, x0[None, :]]
    d = lattice[y0[:, None] + 1, x0[None, :] + 1]
    top = a + (b - a) * fx[None, :]
    bot = c + (d - c) * fx[None, :]
    return top + (bot - top) * fy[:, None]


def ridged(h: int, w: int, *, seed: int = 0, octaves: int = 6,
           base_cell: float = 256.0, gain: float = 2.0, lacunarity: float = 2.0) -> np.ndarray:
    """Ridged multifractal: octave sum of (1-|n|)^2 weighted by the previous octave."""
    rng = np.random.default_rng(seed)
    total = np.zeros((h, w), np.float64)
    weight = np.ones((h, w), np.float64)
    cell = float(base_cell)
    amp = 1.0
    for _ in range(octaves):
        n = _value_noise(h, w, max(cell, 1.0), rng)
        sig = (1.0 - np.abs(n)) ** 2
        sig = sig * weight
        weight = np.clip(sig * gain, 0.0, 1.0)
        total += sig * amp
        cell /= lacunarity
        amp /= lacunarity
    return total


def fbm_ridged(h: int, w: int, *, hurst: float, seed_fbm: int, seed_ridged: int,
               lo: float, hi: float, ridged_weight: float = 0.35) -> np.ndarray:
    base = fbm(h, w, hurst=hurst, seed=seed_fbm, lo=0.0, hi=1.0).astype(np.float64)
    r = ridged(h, w, seed=seed_ridged)
    r = (r - r.min()) / max(r.max() - r.min(), 1e-12)
    return _rescale(base + ridged_weight * r, lo, hi).astype(np.float32)


def nodata_disks(h: int, w: int, *, count: int, seed: int,
                 rmin: float = 10.0, rmax: float = 200.0) -> np.ndarray:
    """Boolean mask of ``count`` seeded disks with radii U(rmin, rmax) px."""
    rng = np.random.default_rng(seed)
    mask = np.zeros((h, w), bool)
    cy = rng.uniform(0, h, count)
    cx = rng.uniform(0, w, count)
    rr = rng.uniform(rmin, rmax, count)
    for y, x, r in zip(cy, cx, rr):
        y0, y1 = max(0, int(y - r) - 1), min(h, int(y + r) + 2)
        x0, x1 = max(0, int(x - r) - 1), min(w, int(x + r) + 2)
        if y0 >= y1 or x0 >= x1:
            continue
        yy, xx = np.mgrid[y0:y1, x0:x1]
        mask[y0:y1, x0:x1] |= (yy - y) ** 2 + (xx - x) ** 2 <= r * r
    return mask


# --------------------------------------------------------------------------- torch
def fbm_device(h: int, w: int, *, hurst: float, seed: int, lo: float, hi: float,
               device="cuda"):
    """fBm with the same spectrum as :func:`fbm`, generated in device memory."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    ky = torch.fft.fftfreq(h, device=device, dtype=torch.float32)[:, None]
    kx = torch.fft.rfftfreq(w, device=device, dtype=torch.float32)[None, :]
    k = torch.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    amp = k.pow_(-(hurst + 1.0))
    amp[0, 0] = 0.0
    spec = torch.complex(torch.randn(amp.shape, generator=g, device=device),
                         torch.randn(amp.shape, generator=g, device=device))
    spec.mul_(amp)
    del amp, k
    field = torch.fft.irfft2(spec, s=(h, w))
    del spec
    fmin = field.min()
    fmax = field.max()
    field.sub_(fmin).mul_((hi - lo) / torch.clamp(fmax - fmin, min=1e-30)).add_(lo)
    return field.to(torch.float32)


def ridged_device(h: int, w: int, *, seed: int, octaves: int = 6, base_cell: float = 256.0,
                  gain: float = 2.0, lacunarity: float = 2.0, device="cuda"):
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    total = torch.zeros((h, w), device=device, dtype=torch.float32)
    weight = torch.ones((h, w), device=device, dtype=torch.float32)
    cell = float(base_cell)
    amp = 1.0
    for _ in range(octaves):
        c = max(cell, 1.0)
        gh = int(math.ceil(h / c)) + 2
        gw = int(math.ceil(w / c)) + 2
        lattice = torch.rand((1, 1, gh, gw), generator=g, device=device) * 2.0 - 1.0
        n = torch.nn.functional.interpolate(
            lattice, size=(int(round(gh * c)), int(round(gw * c))), mode="bicubic",
            align_corners=False)[0, 0, :h, :w]
        sig = (1.0 - n.abs()).pow_(2).mul_(weight)
        weight = torch.clamp(sig * gain, 0.0, 1.0)
        total.add_(sig, alpha=amp)
        del n, sig, lattice
        cell /= lacunarity
        amp /= lacunarity
    return total


def fbm_ridged_device(h: int, w: int, *, hurst: float, seed_fbm: int, seed_ridged: int,
                      lo: float, hi: float, ridged_weight: float = 0.35, device="cuda"):
    base = fbm_device(h, w, hurst=hurst, seed=seed_fbm, lo=0.0, hi=1.0, device=device)
    r = ridged_device(h, w, seed=seed_ridged, device=device)
    rmin, rmax = r.min(), r.max()
    r.sub_(rmin).div_(max(float(rmax - rmin), 1e-12))
    base.add_(r, alpha=ridged_weight)
    del r
    bmin, bmax = base.min(), base.max()
    base.sub_(bmin).mul_((hi - lo) / max(float(bmax - bmin), 1e-30)).add_(lo)
    return base


def nodata_disks_device(dem, *, count: int, seed: int, rmin: float = 10.0,
                        rmax: float = 200.0, value: float = float("nan")):
    """Set ``count`` seeded disks of ``dem`` (a device tensor) to ``value`` in place."""
    import torch

    h, w = dem.shape
    rng = np.random.default_rng(seed)
    cy = rng.uniform(0, h, count)
    cx = rng.uniform(0, w, count)
    rr = rng.uniform(rmin, rmax, count)
    for y, x, r in zip(cy, cx, rr):
        y0, y1 = max(0, int(y - r) - 1), min(h, int(y + r) + 2)
        x0, x1 = max(0, int(x - r) - 1), min(w, int(x + r) + 2)
        if y0 >= y1 or x0 >= x1:
            continue
        yy = torch.arange(y0, y1, device=dem.device, dtype=torch.float32)[:, None]
        xx = torch.arange(x0, x1, device=dem.device, dtype=torch.float32)[None, :]
        m = (yy - y) ** 2 + (xx - x) ** 2 <= r * r
        sub = dem[y0:y1, x0:x1]
        sub.masked_fill_(m, value)
    return dem


def geographic_transform(h: int, w: int, *, lat_top: float = 45.0, lat_bottom: float = 30.0,
                         lon_left: float = 135.0) -> Tuple[float, float, float, float]:
    """(a, e, x0, y0) of an EPSG:4326-style north-up transform: 1 arcsec pixels."""
    a = 1.0 / 3600.0
    e = -(lat_top - lat_bottom) / float(h)
    return a, e, lon_left, lat_top


def nodata_fraction(dem: np.ndarray) -> float:
    return float(np.isnan(dem).mean())


__all__ = [
    "fbm", "ridged", "fbm_ridged", "nodata_disks",
    "fbm_device", "ridged_device", "fbm_ridged_device", "nodata_disks_device",
    "geographic_transform", "nodata_fraction",
]
