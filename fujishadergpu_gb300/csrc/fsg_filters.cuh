// Separable filters shared by topousm_fast, the coarse overview field and the
// spatial-mode smoothing: NaN-aware box means (scipy 'reflect') and Gaussian
// means (scipy 'nearest'), block-mean decimation and corner-aligned bilinear
// zoom.  Reference: algorithms/_nan_utils.py:18-47 and :604-698.
#pragma once

#include "fsg_common.cuh"

namespace fsg {

// scipy.ndimage 'reflect' (half-sample symmetric: d c b a | a b c d | d c b a).
__device__ __forceinline__ int reflect_idx(int k, int n) {
  if (n <= 1) return 0;
  int p = 2 * n;
  int m = k % p;
  if (m < 0) m += p;
  return m < n ? m : p - 1 - m;
}

__device__ __forceinline__ int clamp_idx(int k, int n) { return k < 0 ? 0 : (k >= n ? n - 1 : k); }

// NumPy's pairwise float32 sum of n (<= 16) values x(0..n-1).
template <class Fn>
__device__ __forceinline__ float np_pairwise(int n, Fn x) {
  if (n < 8) {
    float r = 0.f;
    for (int i = 0; i < n; ++i) r = __fadd_rn(r, x(i));
    return r;
  }
  float r[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) r[j] = x(j);
  int i = 8;
  for (; i < n - (n % 8); i += 8)
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = __fadd_rn(r[j], x(i + j));
  float res = __fadd_rn(__fadd_rn(__fadd_rn(r[0], r[1]), __fadd_rn(r[2], r[3])),
                        __fadd_rn(__fadd_rn(r[4], r[5]), __fadd_rn(r[6], r[7])));
  for (; i < n; ++i) res = __fadd_rn(res, x(i));
  return res;
}

// scipy.ndimage.zoom(order=1, mode='nearest', grid_mode=False) of the h x w
// array `a` at zoom-grid point (zy, zx), source coordinate (zy fy, zx fx)
// (zoom1_at), or at any source coordinate (lerp1_at, map_coordinates order 1):
// coordinates and the four-term sum in float64 as scipy computes them, without
// fused multiply-adds, rounded to float32.  nan_aware: the zooms of the NaN -> 0
// values and of the valid mask, each rounded to float32, then num / max(den, 1e-6)
// where den > 1e-3, else NaN (_upsample_to_shape, _nan_utils.py:671-698).
// order-1 spline at the float64 source coordinate (cy, cx), 'nearest' beyond the
// edges (scipy's map_coordinates / zoom arithmetic, shared by both).
__device__ __forceinline__ float lerp1_at(const float* __restrict__ a, long long ld, int h, int w, double cy,
                                          double cx, bool nan_aware) {
  const double sy = floor(cy), sx = floor(cx);
  const double ty = __dsub_rn(cy, sy), tx = __dsub_rn(cx, sx);
  const int iy0 = clamp_idx((int)sy, h), iy1 = clamp_idx((int)sy + 1, h);
  const int ix0 = clamp_idx((int)sx, w), ix1 = clamp_idx((int)sx + 1, w);
  const double wy0 = __dsub_rn(1.0, ty), wx0 = __dsub_rn(1.0, tx);
  const float v00 = __ldg(a + (long long)iy0 * ld + ix0), v01 = __ldg(a + (long long)iy0 * ld + ix1);
  const float v10 = __ldg(a + (long long)iy1 * ld + ix0), v11 = __ldg(a + (long long)iy1 * ld + ix1);
  auto lerp4 = [&](double a00, double a01, double a10, double a11) {
    double t = __dmul_rn(__dmul_rn(a00, wy0), wx0);
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(a01, wy0), tx));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(a10, ty), wx0));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn(a11, ty), tx));
    return __double2float_rn(t);
  };
  if (!nan_aware) return lerp4(v00, v01, v10, v11);
  auto fv = [](float v) { return v == v ? (double)v : 0.0; };
  auto fw = [](float v) { return v == v ? 1.0 : 0.0; };
  const float num = lerp4(fv(v00), fv(v01), fv(v10), fv(v11));
  const float den = lerp4(fw(v00), fw(v01), fw(v10), fw(v11));
  return den > 1e-3f ? __fdiv_rn(num, fmaxf(den, 1e-6f)) : __int_as_float(0x7fc00000);
}
__device__ __forceinline__ float zoom1_at(const float* __restrict__ a, long long ld, int h, int w, int zy, int zx,
                                          double fy, double fx, bool nan_aware) {
  return lerp1_at(a, ld, h, w, __dmul_rn((double)zy, fy), __dmul_rn((double)zx, fx), nan_aware);
}

// Error-free running sum (hi + lo), Knuth's TwoSum.
struct CSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    float s = __fadd_rn(hi, x);
    float bb = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    hi = s;
    lo = __fadd_rn(lo, e);
  }
  __device__ __forceinline__ float value() const { return __fadd_rn(hi, lo); }
};

// View of a float32 raster window with NoData -> NaN applied on load.
struct ZView {
  const float* p;
  long long ld;
  int h, w;
  float ndf;
  int has_nodata;
  __device__ __forceinline__ float at(int y, int x) const {
    float v = __ldg(p + (long long)y * ld + x);
    return is_nodata(v, ndf, has_nodata != 0) ? __int_as_float(0x7fc00000) : v;
  }
};

// Plain float32 array view.
struct AView {
  float* p;
  long long ld;
  int h, w;
  __device__ __forceinline__ float at(int y, int x) const { return p[(long long)y * ld + x]; }
  __device__ __forceinline__ float& ref(int y, int x) const { return p[(long long)y * ld + x]; }
};

}  // namespace fsg
