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
