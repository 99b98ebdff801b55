// Spatial mode of the stencil products: the per-radius smoothing
// _smooth_for_radius (algorithms/_nan_utils.py:527-552) and the pieces of the
// tile backend's per-radius response and weighted combination
// (multiscale_response_fields, _nan_utils.py:441-524).
//
// The smoothing reproduces scipy's arithmetic closely enough that the
// derivative products computed from it stay within float32 rounding of the
// reference (derivatives of a smoothed DEM amplify any error of the
// smoothing):
//   * gaussian_filter: per axis, correlate1d with float64 weights and a
//     float64 accumulator, rounded to float32 after each axis.  Here the
//     accumulation is float-float (~48 bits) on the FP32 pipes and each axis
//     output is rounded once to float32.
//   * the block mean of _downsample_nan_aware sums in NumPy's float32 order:
//     for each row of a cell, NumPy's pairwise sum of the row, added to the
//     running cell total (the reduction over axes (1, 3) of a C-contiguous
//     (oh, f, ow, f) array).
//   * the corner-aligned order-1 zoom interpolates in float64 (as scipy
//     does), summing the four corner terms in scipy's order, then rounds.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "fsg_filters.cuh"

namespace fsg {
namespace {

constexpr int NT = 256;
constexpr float kQNaN = __builtin_nanf("");

// ------------------------------------------------------------ Gaussian
// x * w for a float x and a float-float weight.
__device__ __forceinline__ FF ff_scale(float x, FF w) {
  const float p = __fmul_rn(x, w.hi);
  float e = __fmaf_rn(x, w.hi, -p);
  e = __fmaf_rn(x, w.lo, e);
  return fast_two_sum(p, e);
}

// Symmetric correlate1d at one output: x(0) * w0, then the pairs from the
// outermost inwards, (x(-k) + x(k)) * wk, the order of scipy's symmetric
// branch.  The pair sum is exact as a float-float.
template <class Fn>
__device__ __forceinline__ float corr_ff(const FF* __restrict__ g, int R, Fn x) {
  FF acc = ff_scale(x(0), g[0]);
  for (int k = R; k >= 1; --k) acc = ff_add(acc, ff_mul(two_sum(x(-k), x(k)), g[k]));
  return __fadd_rn(acc.hi, acc.lo);
}

// Axis-0 pass ('nearest'), one output per thread and step: the form for radii
// whose staged lines exceed the shared-memory passes' budget (gauss_axis0_s /
// gauss_axis1_s below take the others).  Channel v: the values (NaN -> 0 when two
// channels are formed); channel w: the valid mask.  Two channels are formed
// when `two` is set, or when *nan_flag is nonzero.
__global__ void __launch_bounds__(NT) gauss_axis0(const float* __restrict__ src, long long ld, int h, int w,
                                                  const FF* __restrict__ g, int R, int two, const int* nan_flag,
                                                  float* v, float* wt, long long old, int rows_per_block) {
  const int x = blockIdx.x * NT + threadIdx.x;
  if (x >= w) return;
  const bool pair = two || (nan_flag != nullptr && *nan_flag != 0);
  const int y0 = blockIdx.y * rows_per_block, y1 = min(h, y0 + rows_per_block);
  for (int y = y0; y < y1; ++y) {
    auto val = [&](int k) {
      const float a = __ldg(src + (long long)clamp_idx(y + k, h) * ld + x);
      return pair ? (a == a ? a : 0.f) : a;
    };
    v[(long long)y * old + x] = corr_ff(g, R, val);
    if (pair) {
      auto ok = [&](int k) {
        const float a = __ldg(src + (long long)clamp_idx(y + k, h) * ld + x);
        return a == a ? 1.f : 0.f;
      };
      wt[(long long)y * old + x] = corr_ff(g, R, ok);
    }
  }
}

enum Axis1Mode { AX1_SMOOTH = 0, AX1_PAIR = 1 };

// Axis-1 pass ('nearest').  AX1_SMOOTH: without NaN in the source (flag 0)
// the filtered values; otherwise where(den > 0, num / den, 0)
// (_nan_utils.py:18-31).  AX1_PAIR: both filtered channels (the void fill).
__global__ void __launch_bounds__(NT) gauss_axis1(const float* __restrict__ v, const float* __restrict__ wt,
                                                  long long ld, int h, int w, const FF* __restrict__ g, int R,
                                                  int mode, const int* nan_flag, float* out, float* out2,
                                                  long long old) {
  const int x = blockIdx.x * NT + threadIdx.x;
  if (x >= w) return;
  const bool pair = mode == AX1_PAIR || (nan_flag != nullptr && *nan_flag != 0);
  for (int y = blockIdx.y; y < h; y += gridDim.y) {
    const float* rv = v + (long long)y * ld;
    const float num = corr_ff(g, R, [&](int k) { return __ldg(rv + clamp_idx(x + k, w)); });
    if (!pair) {
      out[(long long)y * old + x] = num;
      continue;
    }
    const float* rw = wt + (long long)y * ld;
    const float den = corr_ff(g, R, [&](int k) { return __ldg(rw + clamp_idx(x + k, w)); });
    if (mode == AX1_PAIR) {
      out[(long long)y * old + x] = num;
      out2[(long long)y * old + x] = den;
    } else {
      out[(long long)y * old + x] = den > 0.f ? __fdiv_rn(num, den) : 0.f;
    }
  }
}

typedef float2 f2;

// Four consecutive outputs of the symmetric correlate1d along one line, centres
// p0 .. p0+3 of the staged line x(i), each with corr_ff's exact operation
// sequence (so the results are bit-identical to it), as two pairs on the
// paired FP32 instructions.  The accumulations are independent chains, and the
// taps pass between neighbouring outputs: at step k output j pairs x(p0+j-k)
// with x(p0+j+k), and at step k-1 output j's lower tap is output j+1's lower
// tap of step k (upper: output j-1's), so a step loads two values for four
// outputs.
template <class Ld>
__device__ __forceinline__ void corr4_ff(const FF* __restrict__ g, int R, int p0, Ld x, float out[4]) {
  float L[4], U[4];
  const f2 g0h = make_float2(g[0].hi, g[0].hi), g0l = make_float2(g[0].lo, g[0].lo);
  FF2 acc01 = ff_scale2(make_float2(x(p0), x(p0 + 1)), g0h, g0l);
  FF2 acc23 = ff_scale2(make_float2(x(p0 + 2), x(p0 + 3)), g0h, g0l);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    L[j] = x(p0 + j - R);
    U[j] = x(p0 + j + R);
  }
#pragma unroll 2
  for (int k = R; k >= 1; --k) {
    const FF gk = g[k];
    const f2 gh = make_float2(gk.hi, gk.hi), gl = make_float2(gk.lo, gk.lo);
    acc01 = ff_add2(acc01, ff_mul2(two_sum2(make_float2(L[0], L[1]), make_float2(U[0], U[1])), gh, gl));
    acc23 = ff_add2(acc23, ff_mul2(two_sum2(make_float2(L[2], L[3]), make_float2(U[2], U[3])), gh, gl));
    L[0] = L[1];
    L[1] = L[2];
    L[2] = L[3];
    L[3] = x(p0 + 4 - k);
    U[3] = U[2];
    U[2] = U[1];
    U[1] = U[0];
    U[0] = x(p0 + k - 1);
  }
  const f2 o01 = p_add(acc01.hi, acc01.lo), o23 = p_add(acc23.hi, acc23.lo);
  out[0] = o01.x;
  out[1] = o01.y;
  out[2] = o23.x;
  out[3] = o23.y;
}

// Shared-memory forms of the two passes (used while the staged lines fit):
// the weights and the block's source lines (clamped: 'nearest') are staged once,
// and every thread computes four consecutive outputs along the filter axis with
// corr4_ff.  Shared memory layout: weights [R+1] float-float, then the value
// lines, then (two channels) the valid-mask lines.
constexpr int G0C = 32, G0R = 64;   // axis 0: 32 columns x 64 rows; a thread: one column, 2 x 4 rows
constexpr int G1C = 256, G1R = 4;   // axis 1: 4 rows x 256 columns; a thread: one row, 4 columns
constexpr int GNT = 256;
__host__ __device__ constexpr size_t g0_smem(int R) { return 8 * (size_t)(R + 1) + 2 * 4 * (size_t)(G0R + 2 * R) * G0C; }
__host__ __device__ constexpr size_t g1_smem(int R) { return 8 * (size_t)(R + 1) + 2 * 4 * (size_t)G1R * (G1C + 2 * R); }

__global__ void __launch_bounds__(GNT) gauss_axis0_s(const float* __restrict__ src, long long ld, int h, int w,
                                                     const FF* __restrict__ g, int R, int two, const int* nan_flag,
                                                     float* v, float* wt, long long old) {
  extern __shared__ __align__(16) unsigned char gsm[];
  FF* gs = reinterpret_cast<FF*>(gsm);
  float* sv = reinterpret_cast<float*>(gs + R + 1);
  const int rows = G0R + 2 * R;
  float* sw = sv + (size_t)rows * G0C;
  const bool pair = two || (nan_flag != nullptr && *nan_flag != 0);
  const int tid = threadIdx.x, x0 = blockIdx.x * G0C, y0 = blockIdx.y * G0R;
  for (int k = tid; k <= R; k += GNT) gs[k] = g[k];
  for (int i = tid; i < rows * G0C; i += GNT) {
    const int r = i / G0C, c = i - (i / G0C) * G0C;
    const float a = __ldg(src + (long long)clamp_idx(y0 - R + r, h) * ld + min(x0 + c, w - 1));
    if (pair) {
      const bool ok = a == a;
      sv[i] = ok ? a : 0.f;
      sw[i] = ok ? 1.f : 0.f;
    } else {
      sv[i] = a;
    }
  }
  __syncthreads();
  const int c = tid % G0C, x = x0 + c;
#pragma unroll 1
  for (int run = 0; run < 2; ++run) {
    const int r0 = (tid / G0C) * 8 + run * 4;  // block rows r0 .. r0+3
    if (y0 + r0 >= h) break;
    float o[4];
    corr4_ff(gs, R, r0 + R, [&](int i) { return sv[i * G0C + c]; }, o);
    if (x < w)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (y0 + r0 + j < h) v[(long long)(y0 + r0 + j) * old + x] = o[j];
    if (pair) {
      corr4_ff(gs, R, r0 + R, [&](int i) { return sw[i * G0C + c]; }, o);
      if (x < w)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (y0 + r0 + j < h) wt[(long long)(y0 + r0 + j) * old + x] = o[j];
    }
  }
}

__global__ void __launch_bounds__(GNT) gauss_axis1_s(const float* __restrict__ v, const float* __restrict__ wt,
                                                     long long ld, int h, int w, const FF* __restrict__ g, int R,
                                                     int mode, const int* nan_flag, float* out, float* out2,
                                                     long long old) {
  extern __shared__ __align__(16) unsigned char gsm[];
  FF* gs = reinterpret_cast<FF*>(gsm);
  float* sv = reinterpret_cast<float*>(gs + R + 1);
  const int cols = G1C + 2 * R;
  float* sw = sv + (size_t)G1R * cols;
  const bool pair = mode == AX1_PAIR || (nan_flag != nullptr && *nan_flag != 0);
  const int tid = threadIdx.x, x0 = blockIdx.x * G1C, y0 = blockIdx.y * G1R;
  for (int k = tid; k <= R; k += GNT) gs[k] = g[k];
  for (int i = tid; i < G1R * cols; i += GNT) {
    const int r = i / cols, cc = i - (i / cols) * cols;
    const long long off = (long long)min(y0 + r, h - 1) * ld + clamp_idx(x0 - R + cc, w);
    sv[i] = __ldg(v + off);
    if (pair) sw[i] = __ldg(wt + off);
  }
  __syncthreads();
  const int r = tid / (G1C / 4), c0 = 4 * (tid % (G1C / 4)), y = y0 + r;
  if (y >= h) return;
  const float* lv = sv + (size_t)r * cols;
  float num[4];
  corr4_ff(gs, R, c0 + R, [&](int i) { return lv[i]; }, num);
  float* orow = out + (long long)y * old;
  if (!pair) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (x0 + c0 + j < w) orow[x0 + c0 + j] = num[j];
    return;
  }
  const float* lw = sw + (size_t)r * cols;
  float den[4];
  corr4_ff(gs, R, c0 + R, [&](int i) { return lw[i]; }, den);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int x = x0 + c0 + j;
    if (x >= w) continue;
    if (mode == AX1_PAIR) {
      orow[x] = num[j];
      out2[(long long)y * old + x] = den[j];
    } else {
      orow[x] = den[j] > 0.f ? __fdiv_rn(num[j], den[j]) : 0.f;
    }
  }
}

// flag |= any NaN in the h x w array.
__global__ void any_nan(const float* __restrict__ a, long long ld, int h, int w, int* flag) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= w) return;
  bool n = false;
  for (int y = blockIdx.y; y < h; y += gridDim.y) {
    const float v = __ldg(a + (long long)y * ld + x);
    n |= v != v;
  }
  if (__any_sync(__activemask(), n) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// --------------------------------------------------------- decimation
// _downsample_nan_aware's cell mean (_nan_utils.py:629-641): cells padded
// with NaN at the ragged edge, tot / max(cnt, 1) where cnt > 0 else NaN.
__global__ void block_mean_np(const float* __restrict__ src, long long ld, int h, int w, int f, float* out,
                              long long old, int oh, int ow, int* flag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= oh || j >= ow) return;
  float tot = 0.f;
  int cnt = 0;
  for (int a = 0; a < f; ++a) {
    const int y = i * f + a;
    const float* row = src + (long long)min(y, h - 1) * ld;
    auto x = [&](int b) {
      const int xx = j * f + b;
      if (y >= h || xx >= w) return 0.f;
      const float v = __ldg(row + xx);
      return isfinite(v) ? v : 0.f;
    };
    tot = __fadd_rn(tot, np_pairwise(f, x));
    if (y < h)
      for (int b = 0; b < f; ++b) {
        const int xx = j * f + b;
        if (xx < w && isfinite(__ldg(row + xx))) ++cnt;
      }
  }
  const float m = cnt > 0 ? __fdiv_rn(tot, (float)max(cnt, 1)) : kQNaN;
  out[(long long)i * old + j] = m;
  if (m != m) atomicOr(flag, 1);
}

// Enclosed coarse voids: where(nan & sw > 0.5, sv / max(sw, 1e-6), coarse)
// (_nan_utils.py:655-667).
__global__ void void_fill(float* coarse, long long ld, int h, int w, const float* sv, const float* sw,
                          long long sld, const int* flag) {
  if (*flag == 0) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= h || j >= w) return;
  float& c = coarse[(long long)i * ld + j];
  const float ww = sw[(long long)i * sld + j];
  if (c != c && ww > 0.5f) c = __fdiv_rn(sv[(long long)i * sld + j], fmaxf(ww, 1e-6f));
}

// ------------------------------------------------------------ zoom
// scipy.ndimage.zoom(order=1, mode='nearest', grid_mode=False) of an array to
// zh x zw, evaluated over the region [y0, y0+oh) x [x0, x0+ow) of a th x tw
// target with the last row / column repeated where the zoom is smaller
// (_upsample_to_shape, _nan_utils.py:671-698).  Coordinates and the four-term
// sum are float64 as in scipy, without fused multiply-adds.  With NoData in
// the source (*nan_flag != 0; NULL: none) the zoom is NaN-aware: the zooms of
// the NaN -> 0 values and of the valid mask, each rounded to float32, then
// num / max(den, 1e-6) where den > 1e-3, else NaN.
// Launched with 32 x 8 threads, one warp per output row.  Where the block's
// source columns span at most ZL_COLS samples (upsampling), the float64 terms
// that zoom1_at forms per output are shared: the row terms (ty, 1 - ty, source
// rows) come from lane 0, the column terms from warp 0, and the row-weighted
// samples a[iy0][j] * (1 - ty) and a[iy1][j] * ty once per source column j of
// the row; each output then sums its four terms in zoom1_at's order (the same
// roundings, so the same float32).  Other blocks evaluate zoom1_at directly.
constexpr int ZL_COLS = 40;
__global__ void __launch_bounds__(256) zoom_linear(const float* __restrict__ a, long long ld, int h, int w, int zh,
                                                   int zw, double fy, double fx, const int* nan_flag, float* out,
                                                   long long old, int y0, int x0, int oh, int ow) {
  __shared__ double s_tx[32], s_wx[32];
  __shared__ int s_ix0[32], s_ix1[32];
  __shared__ double s_p[8][4][ZL_COLS];  // per row: value rows 0 / 1, mask rows 0 / 1
  const int lane = threadIdx.x, r = threadIdx.y;
  const int x = blockIdx.x * 32 + lane, y = blockIdx.y * 8 + r;
  const bool nan_aware = nan_flag != nullptr && *nan_flag != 0;
  if (r == 0) {
    const int zx = min(x0 + min(x, ow - 1), zw - 1);
    const double cx = __dmul_rn((double)zx, fx), sx = floor(cx);
    const double tx = __dsub_rn(cx, sx);
    s_tx[lane] = tx;
    s_wx[lane] = __dsub_rn(1.0, tx);
    s_ix0[lane] = clamp_idx((int)sx, w);
    s_ix1[lane] = clamp_idx((int)sx + 1, w);
  }
  __syncthreads();
  const int j0 = s_ix0[0], nj = s_ix1[31] - j0 + 1;
  if (nj > ZL_COLS || nj < 1) {  // (uniform over the block) direct evaluation
    if (x < ow && y < oh) {
      const int zy = min(y0 + y, zh - 1), zx = min(x0 + x, zw - 1);
      out[(long long)y * old + x] = zoom1_at(a, ld, h, w, zy, zx, fy, fx, nan_aware);
    }
    return;
  }
  double ty = 0.0, wy = 0.0;
  int iy0 = 0, iy1 = 0;
  if (lane == 0) {
    const int zy = min(y0 + min(y, oh - 1), zh - 1);
    const double cy = __dmul_rn((double)zy, fy), sy = floor(cy);
    ty = __dsub_rn(cy, sy);
    wy = __dsub_rn(1.0, ty);
    iy0 = clamp_idx((int)sy, h);
    iy1 = clamp_idx((int)sy + 1, h);
  }
  ty = __shfl_sync(0xffffffffu, ty, 0);
  wy = __shfl_sync(0xffffffffu, wy, 0);
  iy0 = __shfl_sync(0xffffffffu, iy0, 0);
  iy1 = __shfl_sync(0xffffffffu, iy1, 0);
  for (int j = lane; j < nj; j += 32) {
    const float v0 = __ldg(a + (long long)iy0 * ld + j0 + j), v1 = __ldg(a + (long long)iy1 * ld + j0 + j);
    if (nan_aware) {
      s_p[r][0][j] = __dmul_rn(v0 == v0 ? (double)v0 : 0.0, wy);
      s_p[r][1][j] = __dmul_rn(v1 == v1 ? (double)v1 : 0.0, ty);
      s_p[r][2][j] = __dmul_rn(v0 == v0 ? 1.0 : 0.0, wy);
      s_p[r][3][j] = __dmul_rn(v1 == v1 ? 1.0 : 0.0, ty);
    } else {
      s_p[r][0][j] = __dmul_rn((double)v0, wy);
      s_p[r][1][j] = __dmul_rn((double)v1, ty);
    }
  }
  __syncwarp();
  if (x >= ow || y >= oh) return;
  const int c0 = s_ix0[lane] - j0, c1 = s_ix1[lane] - j0;
  const double tx = s_tx[lane], wx = s_wx[lane];
  auto sum4 = [&](const double* p0, const double* p1) {
    double t = __dmul_rn(p0[c0], wx);
    t = __dadd_rn(t, __dmul_rn(p0[c1], tx));
    t = __dadd_rn(t, __dmul_rn(p1[c0], wx));
    t = __dadd_rn(t, __dmul_rn(p1[c1], tx));
    return __double2float_rn(t);
  };
  float v = sum4(s_p[r][0], s_p[r][1]);
  if (nan_aware) {
    const float den = sum4(s_p[r][2], s_p[r][3]);
    v = den > 1e-3f ? __fdiv_rn(v, fmaxf(den, 1e-6f)) : __int_as_float(0x7fc00000);
  }
  out[(long long)y * old + x] = v;
}

// ------------------------------------------------------ tile pieces
// dask's 'reflect' boundary (the edge sample repeated): index k of a line of
// n samples extended by at most n on each side.
__device__ __forceinline__ int sym_idx(int k, int n) {
  if (k < 0) return -k - 1;
  if (k >= n) return 2 * n - 1 - k;
  return k;
}

__global__ void pad_reflect(ZView z, int y0, int x0, int h, int w, int d, float* dst, long long dld) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w + 2 * d || y >= h + 2 * d) return;
  dst[(long long)y * dld + x] = z.at(y0 + sym_idx(y - d, h), x0 + sym_idx(x - d, w));
}

__global__ void accumulate(const float* __restrict__ src, long long ld, int h, int w, float weight, int first,
                           float* acc, long long ald) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  const float t = __fmul_rn(__ldg(src + (long long)y * ld + x), weight);
  float& o = acc[(long long)y * ald + x];
  o = first ? t : __fadd_rn(o, t);
}

// Element-wise max / min of the stacked responses as NumPy's reductions take
// them: NaN as soon as one operand is NaN.
__global__ void combine_extreme(const float* __restrict__ src, long long ld, int h, int w, int is_max, int first,
                                float* acc, long long ald) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  const float v = __ldg(src + (long long)y * ld + x);
  float& o = acc[(long long)y * ald + x];
  if (first) {
    o = v;
  } else {
    const float a = o;
    o = (a != a || v != v) ? kQNaN : (is_max ? fmaxf(a, v) : fminf(a, v));
  }
}

struct SampleArgs {
  const float* coarse;
  long long cld;
  int ch, cw;
  ZView z;           // raster (NoData mask)
  int y0, x0, h, w;  // region in the raster
  int gy0, gx0;      // global pixel coordinates of the region's first pixel
  float sy, sx;      // f32(ch / full_h), f32(cw / full_w)
  float weight;
  int first;
  float* acc;
  long long ald;
};

// _bilinear_sample_coarse (_nan_utils.py:255-281): float32 coordinates,
// map_coordinates(order=1, mode='nearest') evaluated in float64 and rounded;
// NaN where the raster is NoData (_nan_utils.py:395), then accumulated.
__global__ void sample_coarse(const __grid_constant__ SampleArgs A) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= A.w || y >= A.h) return;
  const int gy = A.gy0 + y, gx = A.gx0 + x;
  const float zv = A.z.at(A.y0 + y, A.x0 + x);
  float v;
  if (zv != zv) {
    v = kQNaN;
  } else {
    const float cy = __fsub_rn(__fmul_rn(__fadd_rn((float)gy, 0.5f), A.sy), 0.5f);
    const float cx = __fsub_rn(__fmul_rn(__fadd_rn((float)gx, 0.5f), A.sx), 0.5f);
    const double dy = (double)cy, dx = (double)cx;
    const double sy = floor(dy), sx = floor(dx);
    const double ty = __dsub_rn(dy, sy), tx = __dsub_rn(dx, sx);
    const int y0 = clamp_idx((int)sy, A.ch), y1 = clamp_idx((int)sy + 1, A.ch);
    const int x0 = clamp_idx((int)sx, A.cw), x1 = clamp_idx((int)sx + 1, A.cw);
    const double wy0 = __dsub_rn(1.0, ty), wx0 = __dsub_rn(1.0, tx);
    const float* C = A.coarse;
    double t = __dmul_rn(__dmul_rn((double)__ldg(C + y0 * A.cld + x0), wy0), wx0);
    t = __dadd_rn(t, __dmul_rn(__dmul_rn((double)__ldg(C + y0 * A.cld + x1), wy0), tx));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn((double)__ldg(C + y1 * A.cld + x0), ty), wx0));
    t = __dadd_rn(t, __dmul_rn(__dmul_rn((double)__ldg(C + y1 * A.cld + x1), ty), tx));
    v = __double2float_rn(t);
  }
  const float tt = __fmul_rn(v, A.weight);
  float& o = A.acc[(long long)y * A.ald + x];
  o = A.first ? tt : __fadd_rn(o, tt);
}

struct StoreArgs {
  const float* acc;
  long long ald;
  ZView z;
  int gy0, gx0, h, w;
  float divisor;            // 1: none
  int mask;                 // NaN at the raster's NoData
  int has_stretch;
  float stretch_lo, stretch_scale;
  void* out;
  long long old;
  int dtype;
  float qa, qb;
  int qmin, qmax;
};

// NaN at the raster's NoData (apply_nodata_mask, core/tile_compute.py:132-152),
// then the plane's encoding.
__global__ void masked_store(const __grid_constant__ StoreArgs A) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= A.w || y >= A.h) return;
  const float zv = A.z.at(A.gy0 + y, A.gx0 + x);
  float v = (A.mask && zv != zv) ? kQNaN : A.acc[(long long)y * A.ald + x];
  if (A.divisor != 1.0f) v = __fdiv_rn(v, A.divisor);
  // apply_display_stretch_dask (_global_stats.py:173-174): max((v - lo) / scale, 0), NaN kept
  if (A.has_stretch && v == v) v = fmaxf(__fdiv_rn(__fsub_rn(v, A.stretch_lo), A.stretch_scale), 0.0f);
  const long long off = (long long)y * A.old + x;
  if (A.dtype == FSG_F32) static_cast<float*>(A.out)[off] = v;
  else if (A.dtype == FSG_U8) static_cast<uint8_t*>(A.out)[off] = (uint8_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
  else static_cast<int16_t*>(A.out)[off] = (int16_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
}

// ------------------------------------------------------------ host
dim3 blocks2d(int h, int w) { return dim3((w + 31) / 32, (h + 7) / 8); }

constexpr size_t kMaxTable = 1 << 16;  // Gaussian weight table bytes (radius <= 8191)
constexpr size_t kStagedSmem = 160 << 10;  // shared-memory Gaussian passes up to this size (radius <= 283)

struct Arena {
  char* p;
  char* end;
  void* take(size_t n) {
    char* q = p;
    p += (n + 255) & ~(size_t)255;
    return p <= end ? q : nullptr;
  }
};

// Gaussian of an h x w array (source and destination may not alias).
// mode AX1_SMOOTH: NaN-aware (checked on the device); AX1_PAIR: the two raw
// channels of where(nan, 0, a) and the valid mask, into dst / dst2.
int gaussian(const float* src, long long ld, int h, int w, double sigma, int mode, float* dst, float* dst2,
             long long dld, Arena& ar, cudaStream_t s) {
  int R;
  std::vector<FF> g = ff_gaussian(sigma, &R);
  if (sizeof(FF) * g.size() > kMaxTable) return fail(FSG_ERR_UNSUPPORTED, "Gaussian radius %d too large", R);
  FF* gd = static_cast<FF*>(ar.take(sizeof(FF) * g.size()));
  float* v = static_cast<float*>(ar.take(sizeof(float) * (size_t)h * w));
  float* wt = static_cast<float*>(ar.take(sizeof(float) * (size_t)h * w));
  int* flag = static_cast<int*>(ar.take(sizeof(int)));
  if (!gd || !v || !wt || !flag) return fail(FSG_ERR_WORKSPACE, "smoothing scratch exhausted");
  FSG_UPLOAD(gd, g.data(), sizeof(FF) * g.size(), s);
  const int* nan_flag = nullptr;
  if (mode == AX1_SMOOTH) {
    FSG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
    any_nan<<<dim3((w + 255) / 256, std::min(h, 1024)), 256, 0, s>>>(src, ld, h, w, flag);
    FSG_LAUNCHED(1);
    nan_flag = flag;
  }
  if (g0_smem(R) <= kStagedSmem && (h + G1R - 1) / G1R <= 65535 && (h + G0R - 1) / G0R <= 65535) {
    static std::mutex attr_mutex;
    static bool attr_set[64] = {};
    int dev = 0;
    FSG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(FSG_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    {
      std::lock_guard<std::mutex> lk(attr_mutex);
      if (!attr_set[dev]) {
        FSG_CUDA(cudaFuncSetAttribute(gauss_axis0_s, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStagedSmem));
        FSG_CUDA(cudaFuncSetAttribute(gauss_axis1_s, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStagedSmem));
        attr_set[dev] = true;
      }
    }
    gauss_axis0_s<<<dim3((w + G0C - 1) / G0C, (h + G0R - 1) / G0R), GNT, g0_smem(R), s>>>(
        src, ld, h, w, gd, R, mode == AX1_PAIR ? 1 : 0, nan_flag, v, wt, w);
    FSG_LAUNCHED(1);
    gauss_axis1_s<<<dim3((w + G1C - 1) / G1C, (h + G1R - 1) / G1R), GNT, g1_smem(R), s>>>(
        v, wt, w, h, w, gd, R, mode, nan_flag, dst, dst2, dld);
    FSG_LAUNCHED(1);
    return FSG_OK;
  }
  const int rpb = 16;
  gauss_axis0<<<dim3((w + NT - 1) / NT, (h + rpb - 1) / rpb), NT, 0, s>>>(
      src, ld, h, w, gd, R, mode == AX1_PAIR ? 1 : 0, nan_flag, v, wt, w, rpb);
  FSG_LAUNCHED(1);
  gauss_axis1<<<dim3((w + NT - 1) / NT, std::min(h, 65535)), NT, 0, s>>>(v, wt, w, h, w, gd, R, mode, nan_flag, dst, dst2, dld);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

// _radius_to_downsample_factor (_nan_utils.py:555-601).
int downsample_factor(double radius, double pixel_size, double algo_factor) {
  const double r = std::max(1.0, radius);
  const double px = std::max(1e-3, pixel_size != 0.0 ? pixel_size : 1.0);
  const double score = (r / 24.0) * algo_factor * 1.0 * std::pow(std::max(1.0, 1.0 / px), 0.35);
  if (score <= 1.0) return 1;
  const double f = std::pow(2.0, std::floor(std::log2(score)));
  return (int)std::max(1.0, std::min(f, 16.0));
}

size_t smooth_scratch_bytes(int h, int w, int f) {
  const size_t full = (size_t)h * w;
  const int hs = (h + f - 1) / f, ws = (w + f - 1) / f;
  const size_t sm = (size_t)hs * ws;
  const size_t gmax = kMaxTable;
  if (f <= 1) return 2 * full * 4 + gmax + 4096;
  return 8 * sm * 4 + 2 * gmax + 8192;
}

}  // namespace
}  // namespace fsg

using namespace fsg;

extern "C" int fsg_smooth(const float* src, int64_t ld, int32_t h, int32_t w, double radius, double pixel_size,
                          double algorithm_factor, float* dst, int64_t dst_ld, void* stream) {
  if (!src || !dst) return fail(FSG_ERR_INVALID, "null array");
  if (h < 0 || w < 0 || ld < w || dst_ld < w) return fail(FSG_ERR_SHAPE, "bad shape %d x %d", h, w);
  if (!(radius == radius) || !(algorithm_factor > 0.0)) return fail(FSG_ERR_INVALID, "bad radius / factor");
  if (h == 0 || w == 0) return FSG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const double r = std::max(1.0, radius);
  if (r <= 1.0) {
    if (src != dst)
      FSG_CUDA(cudaMemcpy2DAsync(dst, dst_ld * 4, src, ld * 4, (size_t)w * 4, h, cudaMemcpyDeviceToDevice, s));
    return FSG_OK;
  }
  const int f = downsample_factor(r, pixel_size, algorithm_factor);
  StreamScratch scratch;
  const size_t bytes = smooth_scratch_bytes(h, w, f);
  int st = scratch.alloc(bytes, s);
  if (st) return st;
  Arena ar{static_cast<char*>(scratch.ptr), static_cast<char*>(scratch.ptr) + bytes};
  if (f <= 1) return gaussian(src, ld, h, w, std::max(0.5, r / 2.0), AX1_SMOOTH, dst, nullptr, dst_ld, ar, s);
  // decimated: NaN-aware block mean (+ enclosed-void fill), Gaussian at the
  // coarse resolution, bilinear zoom back to the block
  const int hs = std::max(1, (h + f - 1) / f), ws = std::max(1, (w + f - 1) / f);
  float* small = static_cast<float*>(ar.take(sizeof(float) * (size_t)hs * ws));
  float* sv = static_cast<float*>(ar.take(sizeof(float) * (size_t)hs * ws));
  float* sw = static_cast<float*>(ar.take(sizeof(float) * (size_t)hs * ws));
  float* sm = static_cast<float*>(ar.take(sizeof(float) * (size_t)hs * ws));
  int* flag = static_cast<int*>(ar.take(sizeof(int)));
  if (!small || !sv || !sw || !sm || !flag) return fail(FSG_ERR_WORKSPACE, "smoothing scratch exhausted");
  FSG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
  block_mean_np<<<blocks2d(hs, ws), dim3(32, 8), 0, s>>>(src, ld, h, w, f, small, ws, hs, ws, flag);
  FSG_LAUNCHED(1);
  // void fill: sigma = max(1, min(shape) / 64); the kernels are cheap when no void exists
  st = gaussian(small, ws, hs, ws, std::max(1.0, (double)std::min(hs, ws) / 64.0), AX1_PAIR, sv, sw, ws, ar, s);
  if (st) return st;
  void_fill<<<blocks2d(hs, ws), dim3(32, 8), 0, s>>>(small, ws, hs, ws, sv, sw, ws, flag);
  FSG_LAUNCHED(1);
  st = gaussian(small, ws, hs, ws, std::max(0.5, (r / f) / 2.0), AX1_SMOOTH, sm, nullptr, ws, ar, s);
  if (st) return st;
  // zoom to round(n * (target / n)) samples per axis, grid_mode=False factors
  const int zh = (int)std::nearbyint((double)hs * ((double)h / (double)hs));
  const int zw = (int)std::nearbyint((double)ws * ((double)w / (double)ws));
  const double fy = zh > 1 ? (double)(hs - 1) / (double)(zh - 1) : 1.0;
  const double fx = zw > 1 ? (double)(ws - 1) / (double)(zw - 1) : 1.0;
  zoom_linear<<<blocks2d(h, w), dim3(32, 8), 0, s>>>(sm, ws, hs, ws, zh, zw, fy, fx, nullptr, dst, dst_ld, 0, 0, h,
                                                     w);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_downsample_nan_aware(const float* src, int64_t ld, int32_t h, int32_t w, int32_t f, float* dst,
                                        int64_t dst_ld, void* stream) {
  if (!src || !dst) return fail(FSG_ERR_INVALID, "null array");
  if (h <= 0 || w <= 0 || ld < w || f < 1) return fail(FSG_ERR_SHAPE, "bad shape %d x %d / factor %d", h, w, f);
  const int hs = (h + f - 1) / f, ws = (w + f - 1) / f;
  if (dst_ld < ws) return fail(FSG_ERR_SHAPE, "destination row too short");
  cudaStream_t s = (cudaStream_t)stream;
  if (f == 1) {
    FSG_CUDA(cudaMemcpy2DAsync(dst, dst_ld * 4, src, ld * 4, (size_t)w * 4, h, cudaMemcpyDeviceToDevice, s));
    return FSG_OK;
  }
  StreamScratch scratch;
  // sv, sw and the Gaussian's two intermediate planes, its table and flags
  const size_t bytes = 6 * (size_t)hs * ws * 4 + 2 * kMaxTable + 8192;
  int st = scratch.alloc(bytes, s);
  if (st) return st;
  Arena ar{static_cast<char*>(scratch.ptr), static_cast<char*>(scratch.ptr) + bytes};
  float* sv = static_cast<float*>(ar.take(sizeof(float) * (size_t)hs * ws));
  float* sw = static_cast<float*>(ar.take(sizeof(float) * (size_t)hs * ws));
  int* flag = static_cast<int*>(ar.take(sizeof(int)));
  if (!sv || !sw || !flag) return fail(FSG_ERR_WORKSPACE, "decimation scratch exhausted");
  FSG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
  block_mean_np<<<blocks2d(hs, ws), dim3(32, 8), 0, s>>>(src, ld, h, w, f, dst, dst_ld, hs, ws, flag);
  FSG_LAUNCHED(1);
  st = gaussian(dst, dst_ld, hs, ws, std::max(1.0, (double)std::min(hs, ws) / 64.0), AX1_PAIR, sv, sw, ws, ar, s);
  if (st) return st;
  void_fill<<<blocks2d(hs, ws), dim3(32, 8), 0, s>>>(dst, dst_ld, hs, ws, sv, sw, ws, flag);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_upsample_to_shape(const float* src, int64_t ld, int32_t h, int32_t w, int32_t th, int32_t tw,
                                     int32_t y0, int32_t x0, int32_t oh, int32_t ow, float* dst, int64_t dst_ld,
                                     void* stream) {
  if (!src || !dst) return fail(FSG_ERR_INVALID, "null array");
  if (h <= 0 || w <= 0 || ld < w || th <= 0 || tw <= 0 || y0 < 0 || x0 < 0 || oh < 0 || ow < 0 || y0 + oh > th ||
      x0 + ow > tw || dst_ld < ow)
    return fail(FSG_ERR_SHAPE, "bad zoom shapes");
  if (oh == 0 || ow == 0) return FSG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch scratch;
  int st = scratch.alloc(256, s);
  if (st) return st;
  int* flag = static_cast<int*>(scratch.ptr);
  FSG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
  any_nan<<<dim3((w + 255) / 256, std::min(h, 1024)), 256, 0, s>>>(src, ld, h, w, flag);
  FSG_LAUNCHED(1);
  // zoom output size round(n * (target / n)) per axis; grid_mode=False factors
  const int zh = (int)std::nearbyint((double)h * ((double)th / (double)h));
  const int zw = (int)std::nearbyint((double)w * ((double)tw / (double)w));
  const double fy = zh > 1 ? (double)(h - 1) / (double)(zh - 1) : 1.0;
  const double fx = zw > 1 ? (double)(w - 1) / (double)(zw - 1) : 1.0;
  zoom_linear<<<blocks2d(oh, ow), dim3(32, 8), 0, s>>>(src, ld, h, w, zh, zw, fy, fx, flag, dst, dst_ld, y0, x0, oh,
                                                       ow);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_pad_reflect(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w, int32_t y0,
                               int32_t x0, int32_t h, int32_t w, int32_t depth, double nodata, int32_t has_nodata,
                               float* dst, int64_t dst_ld, void* stream) {
  if (!raster_dev || !dst) return fail(FSG_ERR_INVALID, "null array");
  if (h <= 0 || w <= 0 || y0 < 0 || x0 < 0 || y0 + h > raster_h || x0 + w > raster_w || ld < raster_w)
    return fail(FSG_ERR_SHAPE, "window [%d, %d) x [%d, %d) outside the %d x %d raster", y0, y0 + h, x0, x0 + w,
                raster_h, raster_w);
  if (depth < 0 || depth > std::min(h, w))
    return fail(FSG_ERR_SHAPE, "reflect depth %d exceeds the window (%d x %d)", depth, h, w);
  if (dst_ld < (int64_t)w + 2 * depth) return fail(FSG_ERR_SHAPE, "destination row too short");
  ZView z{raster_dev, (long long)ld, raster_h, raster_w, (float)nodata, has_nodata};
  pad_reflect<<<blocks2d(h + 2 * depth, w + 2 * depth), dim3(32, 8), 0, (cudaStream_t)stream>>>(
      z, y0, x0, h, w, depth, dst, dst_ld);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_accumulate(const float* src, int64_t ld, int32_t h, int32_t w, float weight, int32_t first,
                              float* acc, int64_t acc_ld, void* stream) {
  if (!src || !acc) return fail(FSG_ERR_INVALID, "null array");
  if (h < 0 || w < 0 || ld < w || acc_ld < w) return fail(FSG_ERR_SHAPE, "bad shape %d x %d", h, w);
  if (h == 0 || w == 0) return FSG_OK;
  accumulate<<<blocks2d(h, w), dim3(32, 8), 0, (cudaStream_t)stream>>>(src, ld, h, w, weight, first, acc, acc_ld);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_combine(const float* src, int64_t ld, int32_t h, int32_t w, int32_t op, float weight,
                           int32_t first, float* acc, int64_t acc_ld, void* stream) {
  if (!src || !acc) return fail(FSG_ERR_INVALID, "null array");
  if (h < 0 || w < 0 || ld < w || acc_ld < w) return fail(FSG_ERR_SHAPE, "bad shape %d x %d", h, w);
  if (op < FSG_COMBINE_WSUM || op > FSG_COMBINE_MIN) return fail(FSG_ERR_INVALID, "unknown combine op %d", op);
  if (h == 0 || w == 0) return FSG_OK;
  if (op == FSG_COMBINE_WSUM)
    accumulate<<<blocks2d(h, w), dim3(32, 8), 0, (cudaStream_t)stream>>>(src, ld, h, w, weight, first, acc, acc_ld);
  else
    combine_extreme<<<blocks2d(h, w), dim3(32, 8), 0, (cudaStream_t)stream>>>(src, ld, h, w,
                                                                              op == FSG_COMBINE_MAX ? 1 : 0, first,
                                                                              acc, acc_ld);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_sample_coarse_accumulate(const float* coarse, int64_t cld, int32_t ch, int32_t cw,
                                            const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                                            int32_t y0, int32_t x0, int32_t h, int32_t w, int64_t gy0, int64_t gx0,
                                            int64_t full_h, int64_t full_w, double nodata, int32_t has_nodata,
                                            float weight, int32_t first, float* acc, int64_t acc_ld, void* stream) {
  if (!coarse || !raster_dev || !acc) return fail(FSG_ERR_INVALID, "null array");
  if (ch <= 0 || cw <= 0 || cld < cw || full_h <= 0 || full_w <= 0) return fail(FSG_ERR_SHAPE, "bad coarse shape");
  if (h < 0 || w < 0 || y0 < 0 || x0 < 0 || y0 + h > raster_h || x0 + w > raster_w || acc_ld < w ||
      ld < raster_w)
    return fail(FSG_ERR_SHAPE, "region outside the raster");
  if (gy0 < 0 || gx0 < 0 || gy0 + h > full_h || gx0 + w > full_w || full_h >= (1 << 24) || full_w >= (1 << 24))
    return fail(FSG_ERR_SHAPE, "global region outside the %lld x %lld raster", (long long)full_h,
                (long long)full_w);
  if (h == 0 || w == 0) return FSG_OK;
  SampleArgs A;
  A.coarse = coarse;
  A.cld = cld;
  A.ch = ch;
  A.cw = cw;
  A.z = ZView{raster_dev, (long long)ld, raster_h, raster_w, (float)nodata, has_nodata};
  A.y0 = y0;
  A.x0 = x0;
  A.gy0 = (int)gy0;
  A.gx0 = (int)gx0;
  A.h = h;
  A.w = w;
  A.sy = (float)((double)ch / (double)full_h);
  A.sx = (float)((double)cw / (double)full_w);
  A.weight = weight;
  A.first = first;
  A.acc = acc;
  A.ald = acc_ld;
  sample_coarse<<<blocks2d(h, w), dim3(32, 8), 0, (cudaStream_t)stream>>>(A);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_masked_store(const float* acc, int64_t acc_ld, const float* raster_dev, int64_t ld,
                                int32_t raster_h, int32_t raster_w, int32_t gy0, int32_t gx0, int32_t h, int32_t w,
                                double nodata, int32_t has_nodata, const fsg_store_finish* finish,
                                const fsg_plane* out, void* stream) {
  if (!acc || !raster_dev || !out || !out->ptr) return fail(FSG_ERR_INVALID, "null array");
  if (finish && !(finish->divisor > 0.0f)) return fail(FSG_ERR_INVALID, "divisor %g", (double)finish->divisor);
  if (h < 0 || w < 0 || gy0 < 0 || gx0 < 0 || gy0 + h > raster_h || gx0 + w > raster_w || acc_ld < w ||
      out->ld < w)
    return fail(FSG_ERR_SHAPE, "region outside the raster");
  if (out->dtype != FSG_F32 && out->dtype != FSG_U8 && out->dtype != FSG_I16)
    return fail(FSG_ERR_DTYPE, "unsupported plane dtype %d", out->dtype);
  if (h == 0 || w == 0) return FSG_OK;
  StoreArgs A;
  A.acc = acc;
  A.ald = acc_ld;
  A.z = ZView{raster_dev, (long long)ld, raster_h, raster_w, (float)nodata, has_nodata};
  A.gy0 = gy0;
  A.gx0 = gx0;
  A.h = h;
  A.w = w;
  A.out = out->ptr;
  A.old = out->ld;
  A.dtype = out->dtype;
  A.qa = out->q_a;
  A.qb = out->q_b;
  A.qmin = out->q_min;
  A.qmax = out->q_max;
  A.divisor = finish ? finish->divisor : 1.0f;
  A.mask = finish ? (finish->keep_nodata_values ? 0 : 1) : 1;
  A.has_stretch = finish && finish->stretch_scale > 1e-12f ? 1 : 0;
  A.stretch_lo = finish ? finish->stretch_lo : 0.0f;
  A.stretch_scale = finish ? finish->stretch_scale : 1.0f;
  masked_store<<<blocks2d(h, w), dim3(32, 8), 0, (cudaStream_t)stream>>>(A);
  FSG_LAUNCHED(1);
  return FSG_OK;
}
