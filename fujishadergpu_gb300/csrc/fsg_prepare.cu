// NoData normalisation and void fill ahead of the hot path: the in-memory form
// of preprocess_dem_to_cog (io/dem_preprocess.py:462-726) without its GDAL /
// COG file I/O.
//
//   fsg_nearest_sample  a nearest-neighbour read of the raster at oh x ow (the
//                       stand-in for GDAL's NEAREST read, :540-546) and its
//                       declared-NoData mask
//   fsg_coarse_average  _nan_aware_coarse_average (:135-188): the k x k cell
//                       mean of the valid samples in NumPy's float32 order,
//                       divided in float64 (float32 sum / int64 count)
//   fsg_pushpull_fill   pushpull_fill (algorithms/_pyramid_fill.py:24-84): the
//                       push levels by scipy's order-1 zoom until every cell
//                       has support, the pull back to full size
//   fsg_edge_connected  _edge_connected_mask (utils/nodata_handler.py:13-25):
//                       4-connected propagation from the border seeds
//   fsg_fill_apply      _apply_band_fill + _sample_coarse (:729-826) over rows
//                       of the full raster: NoData -> NaN, then the bilinear
//                       coarse surface at the pixel's float32 global coordinate
//                       where the fill mode allows
// The coarse grid is small (<= a few thousand px a side); the full-resolution
// pass (fsg_fill_apply) reads and writes each pixel once.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fsg_filters.cuh"

namespace fsg {
namespace {

constexpr int MAX_NODATA_VALUES = 16;

struct NodataSet {
  int n;
  float v[MAX_NODATA_VALUES];  // float32 sentinels compared with ==
};

__device__ __forceinline__ bool in_set(const NodataSet& s, float x) {
  bool hit = false;
  for (int i = 0; i < s.n; ++i) hit |= x == s.v[i];
  return hit;
}

dim3 grid2d(int h, int w) { return dim3((unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8)); }

__global__ void nearest_sample_k(const float* __restrict__ r, long long ld, int h, int w, int oh, int ow, double sy,
                                 double sx, int decl_mode, float ndf, float* __restrict__ out, long long old,
                                 uint8_t* __restrict__ decl, long long dld) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= oh || j >= ow) return;
  // source index trunc((i + 0.5) * (h / oh)) in float64
  const int ys = (int)min((long long)(__dmul_rn((double)i + 0.5, sy)), (long long)h - 1);
  const int xs = (int)min((long long)(__dmul_rn((double)j + 0.5, sx)), (long long)w - 1);
  const float v = __ldg(r + (long long)ys * ld + xs);
  out[(long long)i * old + j] = v;
  // declared NoData: 0 none, 1 NaN, 2 a finite value
  if (decl) decl[(long long)i * dld + j] = decl_mode == 1 ? (v != v) : (decl_mode == 2 ? v == ndf : false);
}

__global__ void coarse_average_k(const float* __restrict__ a, long long ld, const uint8_t* __restrict__ decl,
                                 long long dld, int ch, int cw, int k, NodataSet ns, float* __restrict__ coarse,
                                 long long cld, uint8_t* __restrict__ valid, long long vld, int* any_void) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= ch || j >= cw) return;
  float tot = 0.f;
  long long cnt = 0;
  for (int r = 0; r < k; ++r) {
    const long long y = (long long)i * k + r;
    auto masked = [&](int b) {
      const long long x = (long long)j * k + b;
      const float v = __ldg(a + y * ld + x);
      return (decl && decl[y * dld + x]) || !isfinite(v) || in_set(ns, v);
    };
    tot = __fadd_rn(tot, np_pairwise(k, [&](int b) {
      return masked(b) ? 0.f : __ldg(a + y * ld + (long long)j * k + b);
    }));
    for (int b = 0; b < k; ++b) cnt += masked(b) ? 0 : 1;
  }
  const bool vd = cnt == 0;
  coarse[(long long)i * cld + j] = vd ? 0.f : __double2float_rn(__ddiv_rn((double)tot, (double)cnt));
  valid[(long long)i * vld + j] = vd ? 0 : 1;
  if (vd) atomicOr(any_void, 1);
}

// ---------------------------------------------------------------- push-pull
__global__ void pp_init_k(const float* __restrict__ c, long long cld, const uint8_t* __restrict__ valid,
                          long long vld, int h, int w, float* __restrict__ vw, float* __restrict__ wt) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= h || j >= w) return;
  const bool ok = valid[(long long)i * vld + j] != 0;
  vw[(long long)i * w + j] = ok ? c[(long long)i * cld + j] : 0.f;
  wt[(long long)i * w + j] = ok ? 1.f : 0.f;
}

// One push level: num, den = zoom(vw), zoom(w) to nh x nw; w' = min(den, 1),
// vw' = (den > eps ? num / max(den, eps) : 0) * w'; flag: some w' <= 1e-6.
__global__ void pp_push_k(const float* __restrict__ vw, const float* __restrict__ wt, int h, int w, int nh, int nw,
                          double fy, double fx, float* __restrict__ vw2, float* __restrict__ wt2, int* unsupported) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nh || j >= nw) return;
  const float eps = 1e-6f;
  const float num = zoom1_at(vw, w, h, w, i, j, fy, fx, false);
  const float den = zoom1_at(wt, w, h, w, i, j, fy, fx, false);
  const float wv = fminf(den, 1.0f);
  const float mean = den > eps ? __fdiv_rn(num, fmaxf(den, eps)) : 0.0f;
  vw2[(long long)i * nw + j] = __fmul_rn(mean, wv);
  wt2[(long long)i * nw + j] = wv;
  if ((double)wv <= 1e-6) atomicOr(unsupported, 1);
}

// The apex: filled = w > eps ? vw / max(w, eps) : 0.
__global__ void pp_apex_k(const float* __restrict__ vw, const float* __restrict__ wt, int n, float* __restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float eps = 1e-6f;
  f[i] = wt[i] > eps ? __fdiv_rn(vw[i], fmaxf(wt[i], eps)) : 0.0f;
}

// One pull level: up = zoom(filled fh x fw) to zh x zw, edge-padded / cropped to
// th x tw; filled' = w > eps ? vw / max(w, eps) : up.
__global__ void pp_pull_k(const float* __restrict__ f, int fh, int fw, int zh, int zw, double fy, double fx,
                          const float* __restrict__ vw, const float* __restrict__ wt, int th, int tw,
                          float* __restrict__ f2) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= th || j >= tw) return;
  const float eps = 1e-6f;
  const long long o = (long long)i * tw + j;
  const float wl = wt[o];
  f2[o] = wl > eps ? __fdiv_rn(vw[o], fmaxf(wl, eps))
                   : zoom1_at(f, fw, fh, fw, min(i, zh - 1), min(j, zw - 1), fy, fx, false);
}

__global__ void pp_final_k(const float* __restrict__ c, long long cld, const uint8_t* __restrict__ valid,
                           long long vld, const float* __restrict__ f, int h, int w, int mode, float* __restrict__ out,
                           long long old) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= h || j >= w) return;
  // mode 0: the fill; 1: all valid (copy); 2: none valid (zeros)
  const float cv = c[(long long)i * cld + j];
  float v = cv;
  if (mode == 2) v = 0.f;
  else if (mode == 0) v = valid[(long long)i * vld + j] ? cv : f[(long long)i * w + j];
  out[(long long)i * old + j] = v;
}

// ------------------------------------------------------- edge connectivity
__global__ void edge_seed_k(const uint8_t* __restrict__ m, long long mld, int h, int w, int inv,
                            uint8_t* __restrict__ lab, long long lld) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= h || j >= w) return;
  const bool border = i == 0 || j == 0 || i == h - 1 || j == w - 1;
  lab[(long long)i * lld + j] = (border && ((m[(long long)i * mld + j] != 0) != (inv != 0))) ? 1 : 0;
}

// Propagation inside 32 x 32 tiles until they settle (each pass adds a cell or
// stops, so at most 1024 passes), neighbours across tile edges read from the
// previous state in global memory; `changed` tells the host to launch again.
constexpr int ET = 32;
__global__ void __launch_bounds__(ET * ET) edge_propagate_k(const uint8_t* __restrict__ m, long long mld, int h, int w,
                                                          int inv, uint8_t* lab, long long lld, int* changed) {
  __shared__ uint8_t L[ET + 2][ET + 2];
  __shared__ uint8_t M[ET][ET];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = blockIdx.x * ET + tx, y = blockIdx.y * ET + ty;
  const bool in = x < w && y < h;
  M[ty][tx] = in ? ((m[(long long)y * mld + x] != 0) != (inv != 0)) : 0;
  L[ty + 1][tx + 1] = in ? lab[(long long)y * lld + x] : 0;
  if (ty == 0) {  // halo rows and columns (outside the raster: 0)
    const int xs = blockIdx.x * ET + tx;
    const int yt = blockIdx.y * ET - 1, yb = blockIdx.y * ET + ET;
    L[0][tx + 1] = (xs < w && yt >= 0) ? lab[(long long)yt * lld + xs] : 0;
    L[ET + 1][tx + 1] = (xs < w && yb < h) ? lab[(long long)yb * lld + xs] : 0;
    const int ys = blockIdx.y * ET + tx;
    const int xl = blockIdx.x * ET - 1, xr = blockIdx.x * ET + ET;
    L[tx + 1][0] = (ys < h && xl >= 0) ? lab[(long long)ys * lld + xl] : 0;
    L[tx + 1][ET + 1] = (ys < h && xr < w) ? lab[(long long)ys * lld + xr] : 0;
  }
  __syncthreads();
  bool grew = false;
  for (int pass = 0; pass < ET * ET; ++pass) {
    bool add = false;
    if (M[ty][tx] && !L[ty + 1][tx + 1] &&
        (L[ty][tx + 1] | L[ty + 2][tx + 1] | L[ty + 1][tx] | L[ty + 1][tx + 2]))
      add = true;
    __syncthreads();
    if (add) L[ty + 1][tx + 1] = 1;
    grew |= add;
    if (!__syncthreads_or(add)) break;
  }
  if (in && grew) lab[(long long)y * lld + x] = 1;
  if (__syncthreads_or(grew) && tx == 0 && ty == 0) atomicOr(changed, 1);
}

// ---------------------------------------------------------------- the fill
struct FillArgs {
  const float* raster;
  long long ld;
  int h, w;
  int row0, rows;              // rows [row0, row0 + rows) of the raster
  int decl_mode;               // declared NoData: 0 none, 1 NaN, 2 the value ndf
  float ndf;
  NodataSet extra;             // further sentinels (override, detected)
  int do_fill, fill_all;       // fill NoData; every NoData cell ('all') or not exterior ('enclosed')
  const float* surface;        // ch x cw coarse surface (row pitch sld)
  long long sld;
  const uint8_t* exterior;     // ch x cw exterior mask (nullable)
  long long eld;
  int ch, cw;
  float ry, rx;                // float32(ch / height), float32(cw / width)
  float* out;                  // row r of the range at out + (r - row0) * old
  long long old;
  int* nonfinite;              // set when 'all' leaves a non-finite cell
};

// One pixel of the fill (raster row y, column x, value v).
__device__ __forceinline__ float fill_pixel(const FillArgs& A, int y, int x, float v) {
  const bool declared = A.decl_mode == 1 ? (v != v) : (A.decl_mode == 2 ? v == A.ndf : false);
  const bool wm = declared || !isfinite(v) || in_set(A.extra, v);
  if (!wm) return v;
  v = __int_as_float(0x7fc00000);
  if (A.do_fill) {
    // (row + 0.5) * f32(ch / height) - 0.5 in float32, as _sample_coarse builds it
    const float rr = __fsub_rn(__fmul_rn(__fadd_rn((float)y, 0.5f), A.ry), 0.5f);
    const float cc = __fsub_rn(__fmul_rn(__fadd_rn((float)x, 0.5f), A.rx), 0.5f);
    bool ext = false;
    if (!A.fill_all && A.exterior) {
      // map_coordinates of the 0/1 mask (float32) > 0.5; four equal corners give
      // exactly 0, or 1 within float64 rounding, so only mixed corners are evaluated
      const double cy = (double)rr, cx = (double)cc;
      const double sy = floor(cy), sx = floor(cx);
      const int iy0 = clamp_idx((int)sy, A.ch), iy1 = clamp_idx((int)sy + 1, A.ch);
      const int ix0 = clamp_idx((int)sx, A.cw), ix1 = clamp_idx((int)sx + 1, A.cw);
      const uint8_t* E = A.exterior;
      const int n1 = (E[(long long)iy0 * A.eld + ix0] != 0) + (E[(long long)iy0 * A.eld + ix1] != 0) +
                     (E[(long long)iy1 * A.eld + ix0] != 0) + (E[(long long)iy1 * A.eld + ix1] != 0);
      if (n1 == 4) {
        ext = true;
      } else if (n1 > 0) {
        const double ty = cy - sy, tx = cx - sx;
        auto e = [&](int yy, int xx) { return E[(long long)yy * A.eld + xx] ? 1.0 : 0.0; };
        double t = __dmul_rn(__dmul_rn(e(iy0, ix0), __dsub_rn(1.0, ty)), __dsub_rn(1.0, tx));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(e(iy0, ix1), __dsub_rn(1.0, ty)), tx));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(e(iy1, ix0), ty), __dsub_rn(1.0, tx)));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(e(iy1, ix1), ty), tx));
        ext = __double2float_rn(t) > 0.5f;
      }
    }
    if (!ext) v = lerp1_at(A.surface, A.sld, A.ch, A.cw, (double)rr, (double)cc, false);
  }
  if (!isfinite(v)) {
    if (A.fill_all) atomicOr(A.nonfinite, 1);
    v = __int_as_float(0x7fc00000);
  }
  return v;
}

// One thread per pixel: the NoData pixels' float64 interpolation is a long
// dependent chain on GB300's low-rate FP64 pipe, and as many resident warps as
// possible hide it (a grid-stride variant with four pixels per thread and one
// wave of blocks measured 1.5-1.8x slower).
__global__ void __launch_bounds__(256) fill_apply_k(const __grid_constant__ FillArgs A) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= A.rows || x >= A.w) return;
  const int y = A.row0 + i;
  A.out[(long long)i * A.old + x] = fill_pixel(A, y, x, __ldg(A.raster + (long long)y * A.ld + x));
}

// flags[0] |= some cell invalid, flags[1] |= some cell valid
__global__ void mask_any_k(const uint8_t* __restrict__ m, long long mld, int h, int w, int* flags) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= h || j >= w) return;
  if (m[(long long)i * mld + j]) {
    if (!flags[1]) atomicOr(flags + 1, 1);
  } else if (!flags[0]) {
    atomicOr(flags, 1);
  }
}

// scipy.ndimage.zoom's output length and source step for a zoom of n to about t:
// round(n * (t / n)) and (n - 1) / (out - 1) (1 when out is 1).
void zoom_axis(int n, int t, int* out, double* step) {
  *out = (int)std::nearbyint((double)n * ((double)t / (double)n));
  *step = *out > 1 ? (double)(n - 1) / (double)(*out - 1) : 1.0;
}

// ------------------------------------------------------- value statistics
// Exact value counts for the NoData detection rules (_detect_sentinel_nodata,
// io/dem_preprocess.py:241-275): keys are the float bit patterns with -0 folded
// into +0 (np.unique merges them).  Pass 1 counts the finite, undeclared samples
// per high 16 bits of the order-preserving key and tracks the smallest and
// largest key; pass 2 counts every value of the heavy high-16 bins (those holding at
// least the rule's fraction: at most 1 / fraction of them, MAX_HEAVY in all).
// Equal keys of a warp are merged before their atomic (match.any), so a
// dominant value costs one atomic per warp.
constexpr int MAX_HEAVY = 4096;

__device__ __forceinline__ unsigned order_key(float v) {
  unsigned u = __float_as_uint(v == 0.0f ? 0.0f : v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void value_hist_k(const float* __restrict__ a, long long ld, int h, int w, const uint8_t* __restrict__ decl,
                             long long dld, unsigned* __restrict__ hist, unsigned* kmin, unsigned* kmax) {
  const long long n = (long long)h * w;
  const unsigned lane = threadIdx.x & 31;
  unsigned lo = 0xffffffffu, hi = 0u;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
    const long long i = base + threadIdx.x;
    bool ok = false;
    unsigned k = 0;
    if (i < n) {
      const int y = (int)(i / w), x = (int)(i - (long long)y * w);
      const float v = __ldg(a + (long long)y * ld + x);
      ok = isfinite(v) && !(decl && decl[(long long)y * dld + x]);
      k = order_key(v);
    }
    const unsigned act = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      lo = min(lo, k);
      hi = max(hi, k);
      const unsigned bin = k >> 16;
      const unsigned peers = __match_any_sync(act, bin);
      if ((unsigned)(__ffs(peers) - 1) == lane) atomicAdd(hist + bin, (unsigned)__popc(peers));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) {
    atomicMin(kmin, lo);
    atomicMax(kmax, hi);
  }
}

// slot_of[bin]: the heavy slot of a high-16 bin, or -1
__global__ void value_count_k(const float* __restrict__ a, long long ld, int h, int w,
                             const uint8_t* __restrict__ decl, long long dld, const int* __restrict__ slot_of,
                             unsigned* __restrict__ counts) {
  const long long n = (long long)h * w;
  const unsigned lane = threadIdx.x & 31;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
    const long long i = base + threadIdx.x;
    int slot = -1;
    unsigned k = 0;
    if (i < n) {
      const int y = (int)(i / w), x = (int)(i - (long long)y * w);
      const float v = __ldg(a + (long long)y * ld + x);
      if (isfinite(v) && !(decl && decl[(long long)y * dld + x])) {
        k = order_key(v);
        slot = slot_of[k >> 16];
      }
    }
    const bool ok = slot >= 0;
    const unsigned act = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      const unsigned peers = __match_any_sync(act, k);
      if ((unsigned)(__ffs(peers) - 1) == lane)
        atomicAdd(counts + (size_t)slot * 65536u + (k & 0xffffu), (unsigned)__popc(peers));
    }
  }
}

// number of samples equal (as float32) to v
__global__ void count_equal_k(const float* __restrict__ a, long long ld, int h, int w, float v,
                              unsigned long long* count) {
  const long long n = (long long)h * w;
  unsigned c = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / w), x = (int)(i - (long long)y * w);
    c += __ldg(a + (long long)y * ld + x) == v ? 1u : 0u;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, (unsigned long long)c);
}

int nodata_set(const double* vals, int n, NodataSet* s) {
  if (n < 0 || n > MAX_NODATA_VALUES || (n > 0 && !vals)) return fail(FSG_ERR_INVALID, "bad NoData value list");
  s->n = 0;
  for (int i = 0; i < n; ++i)
    if (std::isfinite(vals[i])) s->v[s->n++] = (float)vals[i];
  return FSG_OK;
}

int read_flag(int* dflag, cudaStream_t s, int* out) {
  FSG_CUDA(cudaMemcpyAsync(out, dflag, sizeof(int), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  return FSG_OK;
}

}  // namespace
}  // namespace fsg

using namespace fsg;

extern "C" int fsg_nearest_sample(const float* raster_dev, int64_t ld, int32_t h, int32_t w, int32_t oh, int32_t ow,
                                  double nodata, int32_t has_nodata, float* sample_dev, int64_t sample_ld,
                                  uint8_t* declared_dev, int64_t declared_ld, void* stream) {
  if (!raster_dev || !sample_dev) return fail(FSG_ERR_INVALID, "null array");
  if (h <= 0 || w <= 0 || ld < w || oh <= 0 || ow <= 0 || sample_ld < ow || (declared_dev && declared_ld < ow))
    return fail(FSG_ERR_SHAPE, "bad sample shapes");
  const int mode = !has_nodata ? 0 : (std::isnan(nodata) ? 1 : 2);
  nearest_sample_k<<<grid2d(oh, ow), dim3(32, 8), 0, (cudaStream_t)stream>>>(
      raster_dev, ld, h, w, oh, ow, (double)h / (double)oh, (double)w / (double)ow, mode, (float)nodata, sample_dev,
      sample_ld, declared_dev, declared_ld);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_coarse_average(const float* sample_dev, int64_t ld, const uint8_t* declared_dev,
                                  int64_t declared_ld, int32_t ch, int32_t cw, int32_t k, const double* nodata_values,
                                  int32_t n_values, float* coarse_dev, int64_t coarse_ld, uint8_t* valid_dev,
                                  int64_t valid_ld, int32_t* any_void, void* stream) {
  if (!sample_dev || !coarse_dev || !valid_dev) return fail(FSG_ERR_INVALID, "null array");
  if (ch <= 0 || cw <= 0 || k < 1 || ld < (int64_t)cw * k || coarse_ld < cw || valid_ld < cw ||
      (declared_dev && declared_ld < (int64_t)cw * k))
    return fail(FSG_ERR_SHAPE, "bad coarse shapes");
  NodataSet ns;
  int st = nodata_set(nodata_values, n_values, &ns);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch flag;
  st = flag.alloc(sizeof(int), s);
  if (st) return st;
  FSG_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int), s));
  coarse_average_k<<<grid2d(ch, cw), dim3(32, 8), 0, s>>>(sample_dev, ld, declared_dev, declared_ld, ch, cw, k, ns,
                                                          coarse_dev, coarse_ld, valid_dev, valid_ld,
                                                          static_cast<int*>(flag.ptr));
  FSG_LAUNCHED(1);
  if (any_void) {
    int v = 0;
    st = read_flag(static_cast<int*>(flag.ptr), s, &v);
    if (st) return st;
    *any_void = v;
  }
  return FSG_OK;
}

extern "C" int fsg_pushpull_fill(const float* coarse_dev, int64_t coarse_ld, const uint8_t* valid_dev,
                                 int64_t valid_ld, int32_t h, int32_t w, float* out_dev, int64_t out_ld,
                                 void* stream) {
  if (!coarse_dev || !valid_dev || !out_dev) return fail(FSG_ERR_INVALID, "null array");
  if (h <= 0 || w <= 0 || coarse_ld < w || valid_ld < w || out_ld < w) return fail(FSG_ERR_SHAPE, "bad shapes");
  cudaStream_t s = (cudaStream_t)stream;
  // level shapes: each a zoom of the previous to max(1, n // 2) per axis, down to 1 x 1
  // (the push stops earlier once every cell of a level has support)
  std::vector<int> lh{h}, lw{w};
  std::vector<double> sy{0.0}, sx{0.0};
  while (std::max(lh.back(), lw.back()) > 1) {
    int zh, zw;
    double fy, fx;
    zoom_axis(lh.back(), std::max(1, lh.back() / 2), &zh, &fy);
    zoom_axis(lw.back(), std::max(1, lw.back() / 2), &zw, &fx);
    lh.push_back(zh);
    lw.push_back(zw);
    sy.push_back(fy);
    sx.push_back(fx);
  }
  std::vector<size_t> off;
  size_t total = 0;
  for (size_t l = 0; l < lh.size(); ++l) {
    off.push_back(total);
    total += ((size_t)lh[l] * lw[l] + 63) & ~(size_t)63;
  }
  const size_t full = ((size_t)h * w + 63) & ~(size_t)63;
  StreamScratch scr;
  int st = scr.alloc(sizeof(float) * (2 * total + 2 * full) + 256, s);
  if (st) return st;
  float* vwb = static_cast<float*>(scr.ptr);
  float* wtb = vwb + total;
  float* fa = wtb + total;
  float* fb = fa + full;
  int* flags = reinterpret_cast<int*>(fb + full);
  FSG_CUDA(cudaMemsetAsync(flags, 0, 2 * sizeof(int), s));
  mask_any_k<<<grid2d(h, w), dim3(32, 8), 0, s>>>(valid_dev, valid_ld, h, w, flags);
  FSG_LAUNCHED(1);
  int hf[2] = {0, 0};
  FSG_CUDA(cudaMemcpyAsync(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  if (!hf[0] || !hf[1]) {  // all valid: the input; none valid: zeros (_pyramid_fill.py:36-40)
    pp_final_k<<<grid2d(h, w), dim3(32, 8), 0, s>>>(coarse_dev, coarse_ld, valid_dev, valid_ld, nullptr, h, w,
                                                     !hf[0] ? 1 : 2, out_dev, out_ld);
    FSG_LAUNCHED(1);
    return FSG_OK;
  }
  pp_init_k<<<grid2d(h, w), dim3(32, 8), 0, s>>>(coarse_dev, coarse_ld, valid_dev, valid_ld, h, w, vwb + off[0],
                                                  wtb + off[0]);
  FSG_LAUNCHED(1);
  // push (:54-65): while the level has more than one cell and some cell lacks support
  size_t top = 0;
  bool unsupported = true;  // level 0 holds an invalid cell
  while (std::max(lh[top], lw[top]) > 1 && unsupported) {
    FSG_CUDA(cudaMemsetAsync(flags, 0, sizeof(int), s));
    pp_push_k<<<grid2d(lh[top + 1], lw[top + 1]), dim3(32, 8), 0, s>>>(
        vwb + off[top], wtb + off[top], lh[top], lw[top], lh[top + 1], lw[top + 1], sy[top + 1], sx[top + 1],
        vwb + off[top + 1], wtb + off[top + 1], flags);
    FSG_LAUNCHED(1);
    int f = 0;
    st = read_flag(flags, s, &f);
    if (st) return st;
    unsupported = f != 0;
    ++top;
  }
  // pull (:67-81)
  const int napex = lh[top] * lw[top];
  pp_apex_k<<<(napex + 255) / 256, 256, 0, s>>>(vwb + off[top], wtb + off[top], napex, fa);
  FSG_LAUNCHED(1);
  float* cur = fa;
  float* nxt = fb;
  int fh = lh[top], fw = lw[top];
  for (size_t l = top; l-- > 0;) {
    const int th = lh[l], tw = lw[l];
    int zh, zw;
    double fy, fx;
    zoom_axis(fh, th, &zh, &fy);
    zoom_axis(fw, tw, &zw, &fx);
    pp_pull_k<<<grid2d(th, tw), dim3(32, 8), 0, s>>>(cur, fh, fw, zh, zw, fy, fx, vwb + off[l], wtb + off[l], th, tw,
                                                      nxt);
    FSG_LAUNCHED(1);
    std::swap(cur, nxt);
    fh = th;
    fw = tw;
  }
  pp_final_k<<<grid2d(h, w), dim3(32, 8), 0, s>>>(coarse_dev, coarse_ld, valid_dev, valid_ld, cur, h, w, 0, out_dev,
                                                   out_ld);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_edge_connected(const uint8_t* mask_dev, int64_t mask_ld, int32_t h, int32_t w, int32_t invert,
                                  uint8_t* out_dev, int64_t out_ld, void* stream) {
  if (!mask_dev || !out_dev) return fail(FSG_ERR_INVALID, "null array");
  if (h <= 0 || w <= 0 || mask_ld < w || out_ld < w) return fail(FSG_ERR_SHAPE, "bad shapes");
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch flag;
  int st = flag.alloc(sizeof(int), s);
  if (st) return st;
  int* changed = static_cast<int*>(flag.ptr);
  edge_seed_k<<<grid2d(h, w), dim3(32, 8), 0, s>>>(mask_dev, mask_ld, h, w, invert, out_dev, out_ld);
  FSG_LAUNCHED(1);
  const dim3 grid((unsigned)((w + ET - 1) / ET), (unsigned)((h + ET - 1) / ET));
  // every launch that reports a change labels at least one more cell
  for (long long it = 0; it <= (long long)h * w; ++it) {
    FSG_CUDA(cudaMemsetAsync(changed, 0, sizeof(int), s));
    edge_propagate_k<<<grid, dim3(ET, ET), 0, s>>>(mask_dev, mask_ld, h, w, invert, out_dev, out_ld, changed);
    FSG_LAUNCHED(1);
    int c = 0;
    st = read_flag(changed, s, &c);
    if (st) return st;
    if (!c) return FSG_OK;
  }
  return fail(FSG_ERR_INVALID, "edge propagation did not settle");
}

extern "C" int fsg_fill_apply(const float* raster_dev, int64_t ld, int32_t h, int32_t w, int32_t row0, int32_t rows,
                              double nodata, int32_t has_nodata, const double* extra_nodata, int32_t n_extra,
                              int32_t fill_mode, const float* surface_dev, int64_t surface_ld,
                              const uint8_t* exterior_dev, int64_t exterior_ld, int32_t ch, int32_t cw,
                              float* out_dev, int64_t out_ld, int32_t* nonfinite, void* stream) {
  if (!raster_dev || !out_dev) return fail(FSG_ERR_INVALID, "null array");
  if (h <= 0 || w <= 0 || ld < w || row0 < 0 || rows < 0 || row0 + rows > h || out_ld < w)
    return fail(FSG_ERR_SHAPE, "bad raster / row range");
  if (fill_mode < FSG_FILL_NONE || fill_mode > FSG_FILL_ALL) return fail(FSG_ERR_INVALID, "fill mode %d", fill_mode);
  const bool do_fill = fill_mode != FSG_FILL_NONE && surface_dev != nullptr;
  if (do_fill && (ch <= 0 || cw <= 0 || surface_ld < cw || (exterior_dev && exterior_ld < cw)))
    return fail(FSG_ERR_SHAPE, "bad coarse surface");
  if (rows == 0) return FSG_OK;
  FillArgs A;
  std::memset(&A, 0, sizeof(A));
  int st = nodata_set(extra_nodata, n_extra, &A.extra);
  if (st) return st;
  A.raster = raster_dev;
  A.ld = ld;
  A.h = h;
  A.w = w;
  A.row0 = row0;
  A.rows = rows;
  A.decl_mode = !has_nodata ? 0 : (std::isnan(nodata) ? 1 : 2);
  A.ndf = (float)nodata;
  A.do_fill = do_fill;
  A.fill_all = fill_mode == FSG_FILL_ALL;
  A.surface = surface_dev;
  A.sld = surface_ld;
  A.exterior = fill_mode == FSG_FILL_ENCLOSED ? exterior_dev : nullptr;
  A.eld = exterior_ld;
  A.ch = ch;
  A.cw = cw;
  A.ry = (float)((double)ch / (double)h);
  A.rx = (float)((double)cw / (double)w);
  A.out = out_dev;
  A.old = out_ld;
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch flag;
  st = flag.alloc(sizeof(int), s);
  if (st) return st;
  A.nonfinite = static_cast<int*>(flag.ptr);
  FSG_CUDA(cudaMemsetAsync(A.nonfinite, 0, sizeof(int), s));
  if ((rows + 7) / 8 > 65535) return fail(FSG_ERR_UNSUPPORTED, "more than 524280 rows in one call");
  timing_mark(s, true);
  fill_apply_k<<<grid2d(rows, w), dim3(32, 8), 0, s>>>(A);
  timing_mark(s, false);
  FSG_LAUNCHED(1);
  if (nonfinite) {
    int v = 0;
    st = read_flag(A.nonfinite, s, &v);
    if (st) return st;
    *nonfinite = v;
  }
  return FSG_OK;
}

extern "C" int fsg_value_mode(const float* sample_dev, int64_t ld, int32_t h, int32_t w, const uint8_t* declared_dev,
                              int64_t declared_ld, double min_fraction, int64_t* n_finite, double* vmin,
                              double* vmax, double* mode_value, int64_t* mode_count, void* stream) {
  if (!sample_dev || !n_finite || !vmin || !vmax || !mode_value || !mode_count)
    return fail(FSG_ERR_INVALID, "null argument");
  if (h <= 0 || w <= 0 || ld < w || (declared_dev && declared_ld < w)) return fail(FSG_ERR_SHAPE, "bad sample shape");
  cudaStream_t s = (cudaStream_t)stream;
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  StreamScratch scr;
  const size_t hist_b = 65536 * sizeof(unsigned);
  st = scr.alloc(hist_b + 65536 * sizeof(int) + 64, s);
  if (st) return st;
  unsigned* hist = static_cast<unsigned*>(scr.ptr);
  int* slot_of = reinterpret_cast<int*>(hist + 65536);
  unsigned* kminmax = reinterpret_cast<unsigned*>(slot_of + 65536);
  const unsigned init[2] = {0xffffffffu, 0u};
  FSG_CUDA(cudaMemsetAsync(hist, 0, hist_b, s));
  FSG_CUDA(cudaMemcpyAsync(kminmax, init, sizeof(init), cudaMemcpyHostToDevice, s));
  const long long n = (long long)h * w;
  const int grid = (int)std::min<long long>((n + 255) / 256, (long long)di.sms * 8);
  value_hist_k<<<grid, 256, 0, s>>>(sample_dev, ld, h, w, declared_dev, declared_ld, hist, kminmax, kminmax + 1);
  FSG_LAUNCHED(1);
  std::vector<unsigned> hh(65536);
  unsigned mm[2];
  FSG_CUDA(cudaMemcpyAsync(hh.data(), hist, hist_b, cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaMemcpyAsync(mm, kminmax, sizeof(mm), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  long long nf = 0;
  for (unsigned c : hh) nf += c;
  *n_finite = nf;
  *mode_count = 0;
  *mode_value = std::nan("");
  *vmin = *vmax = std::nan("");
  if (nf == 0) return FSG_OK;
  auto val = [](unsigned k) {
    const unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    std::memcpy(&f, &u, sizeof(f));
    return (double)f;
  };
  *vmin = val(mm[0]);
  *vmax = val(mm[1]);
  // a value holding at least min_fraction of the samples lies in a bin that does
  std::vector<int> so(65536, -1);
  std::vector<int> heavy;
  for (int b = 0; b < 65536; ++b)
    if (hh[b] > 0 && (double)hh[b] / (double)nf >= min_fraction) {
      if ((int)heavy.size() == MAX_HEAVY) return fail(FSG_ERR_UNSUPPORTED, "min_fraction %g too small", min_fraction);
      so[b] = (int)heavy.size();
      heavy.push_back(b);
    }
  if (heavy.empty()) return FSG_OK;  // no value reaches min_fraction: the mode does not matter
  StreamScratch cscr;  // exact counts of the heavy bins' values
  st = cscr.alloc(heavy.size() * 65536 * sizeof(unsigned), s);
  if (st) return st;
  unsigned* counts = static_cast<unsigned*>(cscr.ptr);
  FSG_CUDA(cudaMemcpyAsync(slot_of, so.data(), 65536 * sizeof(int), cudaMemcpyHostToDevice, s));
  FSG_CUDA(cudaMemsetAsync(counts, 0, heavy.size() * 65536 * sizeof(unsigned), s));
  value_count_k<<<grid, 256, 0, s>>>(sample_dev, ld, h, w, declared_dev, declared_ld, slot_of, counts);
  FSG_LAUNCHED(1);
  std::vector<unsigned> cc(heavy.size() * 65536);
  FSG_CUDA(cudaMemcpyAsync(cc.data(), counts, cc.size() * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  // the most frequent value, the smallest on ties (np.unique + argmax); heavy bins and
  // their low halves ascend with the key, i.e. with the value
  long long best = 0;
  unsigned bestk = 0;
  for (size_t h2 = 0; h2 < heavy.size(); ++h2)
    for (unsigned lo = 0; lo < 65536; ++lo) {
      const unsigned c = cc[h2 * 65536 + lo];
      if ((long long)c > best) {
        best = c;
        bestk = ((unsigned)heavy[h2] << 16) | lo;
      }
    }
  *mode_count = best;
  *mode_value = val(bestk);
  return FSG_OK;
}

extern "C" int fsg_count_equal(const float* sample_dev, int64_t ld, int32_t h, int32_t w, double value,
                               int64_t* count, void* stream) {
  if (!sample_dev || !count) return fail(FSG_ERR_INVALID, "null argument");
  if (h <= 0 || w <= 0 || ld < w) return fail(FSG_ERR_SHAPE, "bad sample shape");
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch scr;
  int st = scr.alloc(sizeof(unsigned long long), s);
  if (st) return st;
  FSG_CUDA(cudaMemsetAsync(scr.ptr, 0, sizeof(unsigned long long), s));
  DeviceInfo di;
  st = device_info(&di);
  if (st) return st;
  const long long n = (long long)h * w;
  const int grid = (int)std::min<long long>((n + 255) / 256, (long long)di.sms * 8);
  count_equal_k<<<grid, 256, 0, s>>>(sample_dev, ld, h, w, (float)value,
                                     static_cast<unsigned long long*>(scr.ptr));
  FSG_LAUNCHED(1);
  unsigned long long c = 0;
  FSG_CUDA(cudaMemcpyAsync(&c, scr.ptr, sizeof(c), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  *count = (int64_t)c;
  return FSG_OK;
}
