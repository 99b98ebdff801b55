// topousm_fast: multiscale box-mean unsharp mask.
//
// Per tile window (algorithms/_impl_topousm_fast.py:49-100 with the tile split
// of algorithms/tile/dask_bridge.py:225-271):
//   for each (small) radius r with weight w:
//     f = downsample factor (_nan_utils.py:555-601, algorithm 'topousm_fast')
//     f > 1 : small = NaN-aware f x f block mean (+ enclosed-void fill),
//             r_s = max(1, round(r/f)); mean_s = box(2r_s+1, reflect) or
//             Gaussian(sigma=1, nearest) if r_s <= 1, both NaN-aware;
//             mean = corner-aligned bilinear zoom of mean_s to the window
//     f == 1: mean = box(2r+1, reflect) (Gaussian(1, nearest) if r <= 1)
//     acc (+)= w * (z - mean)                       (float32, radius order)
//   + large radii: w_large * z - bilinear(coarse field at global coords)
//   / p99 scale, NaN at NoData, optional int16/uint8 encoding of the core.
//
// Box means are separable: a column pass writes float32 vertical means (the
// reference's float32 intermediate) and a row pass, fused with the
// accumulation, consumes them.  Running sums are error-free (TwoSum) so long
// windows do not drift.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <tuple>
#include <vector>

#include "fsg_topousm.cuh"

namespace fsg {
namespace {

constexpr int NT = 256;
constexpr float kQNaN = __builtin_nanf("");

// ----------------------------------------------------------- column passes
// Box: vm = mean over rows [y-r, y+r] of v (NaN -> 0), wm = mean of valid.
template <class Src>
__device__ __forceinline__ void box_cols_body(const Src& src, int r, int chunk, int nan_aware, const AView& vm,
                                              const AView& wm) {
  const int x = blockIdx.x * NT + threadIdx.x;
  if (x >= src.w) return;
  const int y0 = blockIdx.y * chunk;
  const int y1 = min(src.h, y0 + chunk);
  if (y0 >= y1) return;
  const int n = 2 * r + 1;
  const float fn = (float)n;
  CSum s;
  int cnt = 0;
  for (int k = y0 - r; k <= y0 + r; ++k) {
    float v = src.at(reflect_idx(k, src.h), x);
    bool ok = v == v;
    s.add(ok ? v : 0.f);
    cnt += ok;
  }
  for (int y = y0; y < y1; ++y) {
    vm.ref(y, x) = __fdiv_rn(s.value(), fn);
    if (nan_aware) wm.ref(y, x) = __fdiv_rn((float)cnt, fn);
    if (y + 1 < y1) {
      float a = src.at(reflect_idx(y + r + 1, src.h), x);
      float b = src.at(reflect_idx(y - r, src.h), x);
      bool oa = a == a, ob = b == b;
      s.add(oa ? a : 0.f);
      s.add(ob ? -b : -0.f);
      cnt += (int)oa - (int)ob;
    }
  }
}

template <class Src>
__global__ void __launch_bounds__(NT) box_cols(Src src, int r, int chunk, int nan_aware, AView vm, AView wm) {
  box_cols_body(src, r, chunk, nan_aware, vm, wm);
}

// Gaussian column pass (mode 'nearest'): weights g[0..R] (g[0] centre).
template <class Src>
__device__ __forceinline__ void gauss_cols_body(const Src& src, const float* __restrict__ g, int R, int nan_aware,
                                                const AView& vm, const AView& wm) {
  const int x = blockIdx.x * NT + threadIdx.x;
  if (x >= src.w) return;
  for (int y = blockIdx.y; y < src.h; y += gridDim.y) {
  float v0 = src.at(y, x);
  bool o0 = v0 == v0;
  float sv = g[0] * (o0 ? v0 : 0.f);
  float sw = g[0] * (o0 ? 1.f : 0.f);
  for (int k = 1; k <= R; ++k) {
    float a = src.at(clamp_idx(y - k, src.h), x);
    float b = src.at(clamp_idx(y + k, src.h), x);
    bool oa = a == a, ob = b == b;
    sv = fmaf(g[k], __fadd_rn(oa ? a : 0.f, ob ? b : 0.f), sv);
    sw = fmaf(g[k], (float)((int)oa + (int)ob), sw);
  }
  vm.ref(y, x) = sv;
  if (nan_aware) wm.ref(y, x) = sw;
  }
}

template <class Src>
__global__ void __launch_bounds__(NT) gauss_cols(Src src, const float* __restrict__ g, int R, int nan_aware,
                                                 AView vm, AView wm, const int* run_if) {
  if (run_if && *run_if == 0) return;  // nothing to do (e.g. a void fill without voids)
  gauss_cols_body(src, g, R, nan_aware, vm, wm);
}

// ------------------------------------------------------------- row passes
// Output modes of the row pass.
enum RowOut { ROW_MEAN = 0, ROW_ACCUM = 1, ROW_PAIR = 2 };

struct RowArgs {
  AView vm, wm;        // column-pass outputs (wm only if nan_aware)
  int r;               // box radius, or Gaussian radius R
  int nan_aware;
  int gauss;           // 1: Gaussian weights g[0..R] with 'nearest'; 0: box with 'reflect'
  const float* g;
  int mode;            // RowOut
  AView out;           // ROW_MEAN: mean; ROW_ACCUM: acc; ROW_PAIR: numerator
  AView out2;          // ROW_PAIR: denominator
  ZView z;             // ROW_ACCUM: window values
  float weight;
  int first;
  int th, tw;          // tile of outputs per block (th * tw == NT * SEG)
  const int* run_if;   // nullable: skip the pass when *run_if == 0
};

constexpr int SEG = 8;

// shared-memory row of the row pass: column c at c + c / SEG, so the lanes of a
// warp (one SEG-column segment each, SEG = 8 apart) read distinct banks
__device__ __forceinline__ int rp_idx(int c) { return c + c / SEG; }
__host__ __device__ inline int rp_pitch(int span) { return span + span / SEG + 1; }

__device__ __forceinline__ void row_pass_body(const RowArgs& A) {
  extern __shared__ float sm[];
  const int w = A.vm.w, h = A.vm.h;
  const int r = A.r;
  const int span = A.tw + 2 * r, pitch = rp_pitch(span);
  float* sv = sm;
  float* sw = sm + A.th * pitch;
  const int ty0 = blockIdx.y * A.th, tx0 = blockIdx.x * A.tw;
  for (int i = threadIdx.x; i < A.th * span; i += NT) {
    int rr = i / span, c = i - rr * span;
    int y = ty0 + rr;
    if (y >= h) continue;
    int xs = tx0 - r + c;
    int x = A.gauss ? clamp_idx(xs, w) : reflect_idx(xs, w);
    sv[rr * pitch + rp_idx(c)] = A.vm.at(y, x);
    if (A.nan_aware) sw[rr * pitch + rp_idx(c)] = A.wm.at(y, x);
  }
  __syncthreads();
  const int segs_per_row = A.tw / SEG;
  const int rr = threadIdx.x / segs_per_row;
  const int x_begin = tx0 + (threadIdx.x - rr * segs_per_row) * SEG;
  const int y = ty0 + rr;
  if (rr >= A.th || y >= h || x_begin >= w) return;
  const float* rv = sv + rr * pitch;
  const float* rw = sw + rr * pitch;
  auto V = [&](int c) { return rv[rp_idx(c)]; };
  auto Wt = [&](int c) { return rw[rp_idx(c)]; };
  const int n = 2 * r + 1;
  const float fn = (float)n;
  CSum hv, hw;
  const int c0 = x_begin - tx0;  // smem column of x_begin - r
  if (!A.gauss) {
    for (int k = 0; k < n; ++k) {
      hv.add(V(c0 + k));
      if (A.nan_aware) hw.add(Wt(c0 + k));
    }
  }
  for (int j = 0; j < SEG; ++j) {
    const int x = x_begin + j;
    if (x >= w) break;
    float num, den;
    if (A.gauss) {
      const int cc = c0 + j + r;
      float a = A.g[0] * V(cc);
      float b = A.nan_aware ? A.g[0] * Wt(cc) : 0.f;
      for (int k = 1; k <= r; ++k) {
        a = fmaf(A.g[k], __fadd_rn(V(cc - k), V(cc + k)), a);
        if (A.nan_aware) b = fmaf(A.g[k], __fadd_rn(Wt(cc - k), Wt(cc + k)), b);
      }
      num = a;
      den = b;
    } else {
      num = __fdiv_rn(hv.value(), fn);
      den = A.nan_aware ? __fdiv_rn(hw.value(), fn) : 1.f;
      if (j + 1 < SEG) {
        hv.add(V(c0 + j + n));
        hv.add(-V(c0 + j));
        if (A.nan_aware) {
          hw.add(Wt(c0 + j + n));
          hw.add(-Wt(c0 + j));
        }
      }
    }
    if (A.mode == ROW_PAIR) {
      A.out.ref(y, x) = num;
      A.out2.ref(y, x) = den;
      continue;
    }
    float mean = num;
    if (A.nan_aware) mean = den > 0.f ? __fdiv_rn(num, den) : 0.f;
    if (A.mode == ROW_MEAN) {
      A.out.ref(y, x) = mean;
    } else {
      float d = __fmul_rn(A.weight, __fsub_rn(A.z.at(y, x), mean));
      float& acc = A.out.ref(y, x);
      acc = A.first ? d : __fadd_rn(acc, d);
    }
  }
}

__global__ void __launch_bounds__(NT) row_pass(const __grid_constant__ RowArgs A) {
  if (A.run_if && *A.run_if == 0) return;
  row_pass_body(A);
}

// ------------------------------------------------------------ decimation
// NaN-aware f x f block mean (ragged cells padded with NaN); flag |= any NaN.
__global__ void downsample_kernel(ZView z, int f, AView out, int* flag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= out.h || j >= out.w) return;
  float tot = 0.f, cnt = 0.f;
  const int y0 = i * f, x0 = j * f;
  for (int a = 0; a < f; ++a) {
    int y = y0 + a;
    if (y >= z.h) break;
    for (int b = 0; b < f; ++b) {
      int x = x0 + b;
      if (x >= z.w) break;
      float v = z.at(y, x);
      if (isfinite(v)) {
        tot = __fadd_rn(tot, v);
        cnt = __fadd_rn(cnt, 1.f);
      }
    }
  }
  float m = cnt > 0.f ? __fdiv_rn(tot, fmaxf(cnt, 1.f)) : kQNaN;
  out.ref(i, j) = m;
  if (m != m) atomicOr(flag, 1);
}

// _nan_utils.py:655-667: coarse = where(nan & sw > 0.5, sv / max(sw, 1e-6), coarse)
__global__ void voidfill_combine(AView coarse, AView sv, AView sw, const int* flag) {
  if (*flag == 0) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= coarse.h || j >= coarse.w) return;
  float c = coarse.at(i, j);
  float w = sw.at(i, j);
  if (c != c && w > 0.5f) coarse.ref(i, j) = __fdiv_rn(sv.at(i, j), fmaxf(w, 1e-6f));
}

// ---------------------------------------------- batched window decimation
// The decimated radii of all windows of a strip job go through each stage in
// one launch (blockIdx.z = work item: one window and one decimated radius), so
// a stage of a 64-tile raster is one grid of 64x the blocks of one window's
// (the per-window grids are a few dozen blocks and latency-bound).  Per item:
//   small = NaN-aware f x f block mean of the window         (dec_downsample)
//   if small has NaN cells: void fill with the Gaussian gv   (dec_fill_cols, dec_rows 0, dec_fill)
//   ms = box(2 rs + 1, reflect) of small, NaN-aware, or      (dec_mean_cols, dec_rows 1)
//        Gaussian(sigma 1, nearest) when rs <= 1
// The arithmetic is that of the per-window kernels above (decimated_mean).
struct DecItem {
  ZView z;                      // window
  int f, hs, ws;                // decimation factor, decimated grid
  int rs;                       // radius at the decimated resolution
  int R;                        // void-fill Gaussian radius
  const float* gv;              // void-fill weights g[0..R]
  const float* g1;              // sigma-1 weights g[0..4]
  float *small, *vm, *wm, *sw;  // hs x ws scratch (ld = ws)
  float* ms;                    // coarse mean (hs x ws); first the void fill's numerator
  int* flag;                    // any NaN cell in small
  unsigned* zmax;               // nullable: max |z| over the window's valid cells (float bits)
  int* tnan;                    // with zmax: set to 1 when the window holds NoData or a non-finite value
};

__device__ __forceinline__ AView dec_view(float* p, const DecItem& D) { return AView{p, D.ws, D.hs, D.ws}; }

// NaN-aware f x f block means (downsample_kernel) and, for the item that
// carries zmax, the window's max |z| over finite cells (window_absmax's
// quantity, folded into this read of the window).
__global__ void dec_downsample(const DecItem* items) {
  const DecItem& D = items[blockIdx.z];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  float amax = 0.f;
  bool dirty = false;  // NoData or a non-finite value among this thread's cells
  if (i < D.hs && j < D.ws) {
    float tot = 0.f, cnt = 0.f;
    const int y0 = i * D.f, x0 = j * D.f;
    auto take = [&](float v) {  // NoData is NaN here (ZView)
      if (isfinite(v)) {
        tot = __fadd_rn(tot, v);
        cnt = __fadd_rn(cnt, 1.f);
        amax = fmaxf(amax, fabsf(v));
      } else {
        dirty = true;
      }
    };
    const float* p0 = D.z.p + (long long)y0 * D.z.ld + x0;
    // whole cells with 16-byte aligned rows: four columns per load, in the same order
    if ((D.f & 3) == 0 && y0 + D.f <= D.z.h && x0 + D.f <= D.z.w && (D.z.ld & 3) == 0 &&
        (reinterpret_cast<uintptr_t>(p0) & 15) == 0) {
      for (int a = 0; a < D.f; ++a) {
        const float4* r4 = reinterpret_cast<const float4*>(p0 + (long long)a * D.z.ld);
        for (int b = 0; b < D.f / 4; ++b) {
          const float4 v = __ldg(r4 + b);
          const bool h = D.z.has_nodata != 0;
          take(is_nodata(v.x, D.z.ndf, h) ? kQNaN : v.x);
          take(is_nodata(v.y, D.z.ndf, h) ? kQNaN : v.y);
          take(is_nodata(v.z, D.z.ndf, h) ? kQNaN : v.z);
          take(is_nodata(v.w, D.z.ndf, h) ? kQNaN : v.w);
        }
      }
    } else {
      for (int a = 0; a < D.f; ++a) {
        const int y = y0 + a;
        if (y >= D.z.h) break;
        for (int b = 0; b < D.f; ++b) {
          const int x = x0 + b;
          if (x >= D.z.w) break;
          take(D.z.at(y, x));
        }
      }
    }
    const float m = cnt > 0.f ? __fdiv_rn(tot, fmaxf(cnt, 1.f)) : kQNaN;
    D.small[(long long)i * D.ws + j] = m;
    if (m != m) atomicOr(D.flag, 1);
  }
  if (D.zmax) {  // block-uniform: block maximum, one atomic only where it raises the running value
    if (__syncthreads_or(dirty) && threadIdx.x == 0 && threadIdx.y == 0) *D.tnan = 1;
    __shared__ float wmax[8];
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    if ((t & 31) == 0) wmax[t >> 5] = amax;
    __syncthreads();
    if (t == 0) {
      float m = wmax[0];
      for (int w = 1; w < (int)((blockDim.x * blockDim.y) >> 5); ++w) m = fmaxf(m, wmax[w]);
      // the running value only grows, so a stale read can only let a redundant atomic through
      if (m > 0.f && m > __uint_as_float(*reinterpret_cast<volatile unsigned*>(D.zmax)))
        atomicMax(D.zmax, __float_as_uint(m));
    }
  }
}

// Void fill, column pass: Gaussian(gv, nearest) of small -> vm, wm.
__global__ void __launch_bounds__(NT) dec_fill_cols(const DecItem* items) {
  const DecItem& D = items[blockIdx.z];
  if (*D.flag == 0 || blockIdx.x * NT >= D.ws) return;
  gauss_cols_body(dec_view(D.small, D), D.gv, D.R, 1, dec_view(D.vm, D), dec_view(D.wm, D));
}

// Row passes. stage 0: void fill, Gaussian(gv) rows of vm, wm -> numerator (ms),
// denominator (sw); stage 1: the mean of the radius, rows of vm, wm -> ms.
__global__ void __launch_bounds__(NT) dec_rows(const DecItem* items, int stage, int th, int tw) {
  const DecItem& D = items[blockIdx.z];
  if ((stage == 0 && *D.flag == 0) || blockIdx.x * tw >= D.ws || blockIdx.y * th >= D.hs) return;
  RowArgs A;
  A.vm = dec_view(D.vm, D);
  A.wm = dec_view(D.wm, D);
  A.nan_aware = 1;
  A.th = th;
  A.tw = tw;
  A.run_if = nullptr;
  A.weight = 0.f;
  A.first = 0;
  A.z = D.z;
  A.out2 = dec_view(D.sw, D);
  A.out = dec_view(D.ms, D);
  if (stage == 0) {
    A.mode = ROW_PAIR;
    A.gauss = 1;
    A.r = D.R;
    A.g = D.gv;
  } else {
    A.mode = ROW_MEAN;
    A.gauss = D.rs <= 1;
    A.r = D.rs <= 1 ? 4 : D.rs;
    A.g = D.g1;
  }
  row_pass_body(A);
}

// _nan_utils.py:655-667 (voidfill_combine): small = where(nan & sw > 0.5, sv / max(sw, 1e-6), small)
__global__ void dec_fill(const DecItem* items) {
  const DecItem& D = items[blockIdx.z];
  if (*D.flag == 0) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= D.ws) return;
  for (int i = blockIdx.y * blockDim.y + threadIdx.y; i < D.hs; i += gridDim.y * blockDim.y) {
    const long long o = (long long)i * D.ws + j;
    const float c = D.small[o], w = D.sw[o];
    if (c != c && w > 0.5f) D.small[o] = __fdiv_rn(D.ms[o], fmaxf(w, 1e-6f));
  }
}

// Column pass of the radius's mean: box(2 rs + 1, reflect) or Gaussian(sigma 1, nearest).
__global__ void __launch_bounds__(NT) dec_mean_cols(const DecItem* items, int chunk) {
  const DecItem& D = items[blockIdx.z];
  if (blockIdx.x * NT >= D.ws) return;
  if (D.rs <= 1) {
    gauss_cols_body(dec_view(D.small, D), D.g1, 4, 1, dec_view(D.vm, D), dec_view(D.wm, D));
  } else {
    if (blockIdx.y * chunk >= D.hs) return;
    box_cols_body(dec_view(D.small, D), D.rs, chunk, 1, dec_view(D.vm, D), dec_view(D.wm, D));
  }
}

// ------------------------------------------------------------- upsample
// acc (+)= w * (z - zoom(mean_s)), scipy zoom order 1, grid_mode False
// (corner-aligned: in = out * (n_in - 1) / (n_out - 1)), mode 'nearest'.
__global__ void accum_upsample(ZView z, AView ms, double zy, double zx, float weight, int first, AView acc) {
  __shared__ int iy0[32], iy1[32];
  __shared__ float fy[32];
  __shared__ int ix0[32], ix1[32];
  __shared__ float fx[32];
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  const int bx0 = blockIdx.x * 32, by0 = blockIdx.y * 32;
  const int lin = ty * 32 + tx;
  if (lin < 32) {
    int o = by0 + lin;
    double c = (double)o * zy;
    int s = (int)floor(c);
    fy[lin] = (float)(c - (double)s);
    iy0[lin] = clamp_idx(s, ms.h);
    iy1[lin] = clamp_idx(s + 1, ms.h);
  } else if (lin < 64) {
    int k = lin - 32;
    int o = bx0 + k;
    double c = (double)o * zx;
    int s = (int)floor(c);
    fx[k] = (float)(c - (double)s);
    ix0[k] = clamp_idx(s, ms.w);
    ix1[k] = clamp_idx(s + 1, ms.w);
  }
  __syncthreads();
  const int x = bx0 + tx;
  if (x >= z.w) return;
  for (int k = ty; k < 32; k += 8) {
    const int y = by0 + k;
    if (y >= z.h) break;
    float a = ms.at(iy0[k], ix0[tx]), b = ms.at(iy0[k], ix1[tx]);
    float c = ms.at(iy1[k], ix0[tx]), d = ms.at(iy1[k], ix1[tx]);
    float top = fmaf(fx[tx], b - a, a);
    float bot = fmaf(fx[tx], d - c, c);
    float mean = fmaf(fy[k], bot - top, top);
    float dd = __fmul_rn(weight, __fsub_rn(z.at(y, x), mean));
    float& o = acc.ref(y, x);
    o = first ? dd : __fadd_rn(o, dd);
  }
}

// --------------------------------------------------------------- final
struct FinalArgs {
  ZView z;             // window
  AView acc;           // small-radius sum (valid if have_small)
  int have_small;
  const float* field;  // coarse field (nullable)
  long long fld;
  int fh, fw;
  float sy, sx;        // f32(ch / full_h), f32(cw / full_w)
  float w_large;
  int gy0, gx0;        // global coords of the window origin
  int cy0, cx0, ch, cw;  // core, window coords
  float scale;         // 0: raw
  void* out;
  long long old;
  int dtype;
  float qa, qb;
  int qmin, qmax;
};

__device__ __forceinline__ float field_sample(const FinalArgs& A, int gy, int gx) {
  // _nan_utils.py:276-281: coords in float32, map_coordinates order 1, 'nearest'.
  float cy = __fsub_rn(__fmul_rn(__fadd_rn((float)gy, 0.5f), A.sy), 0.5f);
  float cx = __fsub_rn(__fmul_rn(__fadd_rn((float)gx, 0.5f), A.sx), 0.5f);
  float fy0 = floorf(cy), fx0 = floorf(cx);
  float ty = cy - fy0, tx = cx - fx0;
  int y0 = clamp_idx((int)fy0, A.fh), y1 = clamp_idx((int)fy0 + 1, A.fh);
  int x0 = clamp_idx((int)fx0, A.fw), x1 = clamp_idx((int)fx0 + 1, A.fw);
  const float* F = A.field;
  float a = __ldg(F + y0 * A.fld + x0), b = __ldg(F + y0 * A.fld + x1);
  float c = __ldg(F + y1 * A.fld + x0), d = __ldg(F + y1 * A.fld + x1);
  float top = fmaf(tx, b - a, a);
  float bot = fmaf(tx, d - c, c);
  return fmaf(ty, bot - top, top);
}

__global__ void final_kernel(const __grid_constant__ FinalArgs A) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= A.cw || y >= A.ch) return;
  const int wy = A.cy0 + y, wx = A.cx0 + x;
  float zv = A.z.at(wy, wx);
  float v;
  if (zv != zv) {
    v = kQNaN;
  } else {
    float large = 0.f;
    bool have_large = A.field != nullptr;
    if (have_large) large = __fsub_rn(__fmul_rn(A.w_large, zv), field_sample(A, A.gy0 + wy, A.gx0 + wx));
    if (A.have_small) v = have_large ? __fadd_rn(A.acc.at(wy, wx), large) : A.acc.at(wy, wx);
    else v = large;
    if (A.scale > 0.f) v = __fdiv_rn(v, A.scale);
  }
  long long off = (long long)y * A.old + x;
  if (A.dtype == FSG_F32) {
    static_cast<float*>(A.out)[off] = v;
  } else if (A.dtype == FSG_U8) {
    static_cast<uint8_t*>(A.out)[off] = (uint8_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
  } else {
    static_cast<int16_t*>(A.out)[off] = (int16_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
  }
}

// Coarse field accumulation: field (+)= f32(w) * mean (_impl_topousm_fast.py:153-154).
__global__ void field_accum(AView mean, float w, int first, AView field) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= mean.w || y >= mean.h) return;
  float t = __fmul_rn(w, mean.at(y, x));
  float& f = field.ref(y, x);
  f = first ? t : __fadd_rn(f, t);
}

// Overview decimation: NaN-aware mean of the source pixels whose centres fall
// in each output cell (an exact f x f block mean for integer factors).  The
// sum is float-float (about 48 significant bits; GB300's FP64 rate is a small
// fraction of its FP32 rate) in four independent chains, the mean formed in
// double once per cell.
__global__ void overview_kernel(ZView z, AView out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= out.h || j >= out.w) return;
  const int ya = (int)(((long long)i * z.h) / out.h), yb = (int)(((long long)(i + 1) * z.h) / out.h);
  const int xa = (int)(((long long)j * z.w) / out.w), xb = (int)(((long long)(j + 1) * z.w) / out.w);
  FF acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  int cnt = 0;
  auto add4 = [&](const float (&v)[4]) {
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      if (!is_nodata(v[m], z.ndf, z.has_nodata != 0)) {
        const FF t = two_sum(acc[m].hi, v[m]);
        acc[m] = {t.hi, __fadd_rn(acc[m].lo, t.lo)};
        ++cnt;
      }
    }
  };
  // 16-byte loads when the cell's rows start aligned (same chains, same order)
  const bool vec = (z.ld & 3) == 0 && (reinterpret_cast<uintptr_t>(z.p + xa) & 15) == 0;
  for (int y = ya; y < yb; ++y) {
    const float* row = z.p + (long long)y * z.ld;
    int x = xa;
    if (vec) {
      for (; x + 3 < xb; x += 4) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(row + x));
        const float v[4] = {q.x, q.y, q.z, q.w};
        add4(v);
      }
    }
    for (; x + 3 < xb; x += 4) {
      const float v[4] = {__ldg(row + x), __ldg(row + x + 1), __ldg(row + x + 2), __ldg(row + x + 3)};
      add4(v);
    }
    for (; x < xb; ++x) {
      const float v = __ldg(row + x);
      if (!is_nodata(v, z.ndf, z.has_nodata != 0)) {
        const FF t = two_sum(acc[0].hi, v);
        acc[0] = {t.hi, __fadd_rn(acc[0].lo, t.lo)};
        ++cnt;
      }
    }
  }
  double tot = 0.0;
#pragma unroll
  for (int m = 0; m < 4; ++m) tot += (double)acc[m].hi + (double)acc[m].lo;
  out.ref(i, j) = cnt ? (float)(tot / (double)cnt) : kQNaN;
}

// ------------------------------------------------ fused full-resolution pass
// All full-resolution box radii (downsample factor 1, r >= 2) of a tile in one
// pass, then the rest of the output in the reference's order.  A CTA owns a
// strip of TW = 256 - 2R output columns (R = largest such radius) and a chunk
// of rows.  Each thread keeps one buffer column's running vertical sums
// (compensated, per radius; 'reflect' rows) in registers and writes that
// column's vertical means (the float32 intermediate of uniform_filter's first
// axis) for G rows into shared memory; the horizontal means are running sums
// over SEG-column segments of those rows (the buffer already holds the
// reflected columns).  The epilogue adds the decimated radii (bilinear zoom of
// their coarse means, as accum_upsample), the large-radius field, the scale and
// the encoding, and stores each output pixel once.
// shared-memory row of ST_NT buffer columns; column c lives at c + c / 8 so
// that threads walking 8-column segments hit distinct banks
constexpr int ST_ROW = ST_NT + ST_NT / 8;
__device__ __forceinline__ int sidx(int c) { return c + (c >> 3); }

__device__ __forceinline__ float field_at(const StripArgs& A, int gy, int gx) {
  // _nan_utils.py:276-281: coords in float32, map_coordinates order 1, 'nearest' (as field_sample).
  float cy = __fsub_rn(__fmul_rn(__fadd_rn((float)gy, 0.5f), A.sy), 0.5f);
  float cx = __fsub_rn(__fmul_rn(__fadd_rn((float)gx, 0.5f), A.sx), 0.5f);
  float fy0 = floorf(cy), fx0 = floorf(cx);
  float ty = cy - fy0, tx = cx - fx0;
  int y0 = clamp_idx((int)fy0, A.fh), y1 = clamp_idx((int)fy0 + 1, A.fh);
  int x0 = clamp_idx((int)fx0, A.fw), x1 = clamp_idx((int)fx0 + 1, A.fw);
  const float* F = A.field;
  float a = __ldg(F + y0 * A.fld + x0), b = __ldg(F + y0 * A.fld + x1);
  float c = __ldg(F + y1 * A.fld + x0), d = __ldg(F + y1 * A.fld + x1);
  float top = fmaf(tx, b - a, a);
  float bot = fmaf(tx, d - c, c);
  return fmaf(ty, bot - top, top);
}



// Shared memory of the strip kernel (floats):
//   V  [G][nr][2][ST_ROW]  vertical means (values, valid fraction), padded columns
//   M  [G][nr][TW + TW/16 + 1] horizontal means per radius, padded columns
//   DY [ST_MAXD][G] (int y0, int y1, float fy)   decimated-grid row coordinates of the G rows
//   DX [ST_MAXD][TW] (int x0, int x1, float fx)  decimated-grid column coordinates of the strip
struct StripSmem {
  static size_t floats(int nr, int TW) {
    return (size_t)ST_G * nr * 2 * ST_ROW + (size_t)ST_G * nr * (TW + TW / 16 + 1) + 3 * (size_t)ST_MAXD * ST_G +
           3 * (size_t)ST_MAXD * TW;
  }
};

constexpr int ST_HSEG = 16;  // columns per horizontal running-sum segment
// horizontal-mean row: column j at j + j / 16 (segment walks hit distinct banks)
__device__ __forceinline__ int midx(int j) { return j + (j >> 4); }

template <int NR>
__global__ void __launch_bounds__(ST_NT) topousm_strip(const __grid_constant__ StripArgs A) {
  extern __shared__ float smem[];
  constexpr int nr = NR;
  const int TW = A.TW;
  const int MROW = TW + TW / ST_HSEG + 1;
  float* V = smem;
  float* M = V + (size_t)ST_G * nr * 2 * ST_ROW;
  int* DYi = reinterpret_cast<int*>(M + (size_t)ST_G * nr * MROW);  // [ST_MAXD][G][2]
  float* DYf = reinterpret_cast<float*>(DYi + 2 * ST_MAXD * ST_G);  // [ST_MAXD][G]
  int* DXi = reinterpret_cast<int*>(DYf + ST_MAXD * ST_G);          // [ST_MAXD][TW][2]
  float* DXf = reinterpret_cast<float*>(DXi + 2 * ST_MAXD * TW);    // [ST_MAXD][TW]
  const int b = threadIdx.x;  // buffer column of the vertical pass
  // the item's tile descriptor, staged in shared memory: the output stores
  // could alias a global copy as far as the compiler knows
  __shared__ TopoTileK Ts;
  const TopoTileK& T = Ts;
  for (int it = blockIdx.x; it < A.nitems; it += gridDim.x) {
    const StripItem I = A.items[it];
    __syncthreads();
    for (int k = threadIdx.x; k < (int)(sizeof(TopoTileK) / 4); k += ST_NT)
      reinterpret_cast<int*>(&Ts)[k] = reinterpret_cast<const int*>(A.tiles + I.tile)[k];
    __syncthreads();
    const bool nanw = *T.nan_flag != 0;
    const ZView& z = T.z;
    const int xc = reflect_idx(I.x0 - A.R + b, z.w);  // window column of this buffer column
    const int xend = min(I.x0 + TW, T.cx0 + T.cw);     // end of the strip's outputs
    // every row the vertical sums enter or leave lies inside the window
    const bool rows_inside = I.y0 - A.R >= 0 && I.y1 + A.R < z.h;
    // decimated-grid column coordinates of the strip (accum_upsample's zoom)
    for (int d = 0; d < T.ndec; ++d)
      for (int j = threadIdx.x; j < TW; j += ST_NT) {
        const DecK& D = T.dec[d];
        const double c = (double)(I.x0 + j) * D.zx;
        const int sx = (int)floor(c);
        DXi[(d * TW + j) * 2] = clamp_idx(sx, D.w);
        DXi[(d * TW + j) * 2 + 1] = clamp_idx(sx + 1, D.w);
        DXf[d * TW + j] = (float)(c - (double)sx);
      }
    CSum vs[NR > 0 ? NR : 1];
    int vc[NR > 0 ? NR : 1];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      vc[q] = 0;
      const int r = A.radii[q];
      for (int k = -r; k <= r; ++k) {
        const float v = z.at(reflect_idx(I.y0 + k, z.h), xc);
        const bool ok = v == v;
        vs[q].add(ok ? v : 0.f);
        vc[q] += ok;
      }
    }
    for (int yg = I.y0; yg < I.y1; yg += ST_G) {
      const int gn = min(ST_G, I.y1 - yg);
      // (1) vertical means of the group's rows, then slide the sums; the rows
      //     entering and leaving the windows are loaded for the whole group first
      if (NR > 0) {
        float za[ST_G][NR > 0 ? NR : 1], zc[ST_G][NR > 0 ? NR : 1];
        if (rows_inside) {  // no reflection anywhere in this chunk (uniform branch)
          const float* col = z.p + xc;
#pragma unroll
          for (int i = 0; i < ST_G; ++i)
#pragma unroll
            for (int q = 0; q < NR; ++q) {
              const int r = A.radii[q];
              const int y = min(yg + i, I.y1 - 1);
              float a = __ldg(col + (long long)(y + r + 1) * z.ld), c = __ldg(col + (long long)(y - r) * z.ld);
              if (z.has_nodata) {
                if (is_nodata(a, z.ndf, true)) a = kQNaN;
                if (is_nodata(c, z.ndf, true)) c = kQNaN;
              }
              za[i][q] = a;
              zc[i][q] = c;
            }
        } else {
#pragma unroll
          for (int i = 0; i < ST_G; ++i)
#pragma unroll
            for (int q = 0; q < NR; ++q) {
              const int r = A.radii[q];
              const int y = min(yg + i, I.y1 - 1);
              za[i][q] = z.at(reflect_idx(y + r + 1, z.h), xc);
              zc[i][q] = z.at(reflect_idx(y - r, z.h), xc);
            }
        }
#pragma unroll
        for (int i = 0; i < ST_G; ++i) {
          if (i >= gn) break;
#pragma unroll
          for (int q = 0; q < NR; ++q) {
            float* vrow = V + ((i * nr + q) * 2) * ST_ROW;
            vrow[sidx(b)] = div_by(vs[q].value(), A.fn[q], A.rn[q]);
            if (nanw) vrow[ST_ROW + sidx(b)] = div_by((float)vc[q], A.fn[q], A.rn[q]);
            const float a = za[i][q], c = zc[i][q];
            const bool oa = a == a, oc = c == c;
            vs[q].add(oa ? a : 0.f);
            vs[q].add(oc ? -c : -0.f);
            vc[q] += (int)oa - (int)oc;
          }
        }
      }
      if (threadIdx.x < T.ndec * ST_G) {  // decimated-grid row coordinates of the group
        const int d = threadIdx.x / ST_G, i = threadIdx.x - (threadIdx.x / ST_G) * ST_G;
        const DecK& D = T.dec[d];
        const double c = (double)(yg + i) * D.zy;
        const int sy = (int)floor(c);
        DYi[(d * ST_G + i) * 2] = clamp_idx(sy, D.h);
        DYi[(d * ST_G + i) * 2 + 1] = clamp_idx(sy + 1, D.h);
        DYf[d * ST_G + i] = (float)(c - (double)sy);
      }
      __syncthreads();
      // (2) horizontal means: task = (row, radius, 16-column segment)
      const int nseg = (TW + ST_HSEG - 1) / ST_HSEG;
      // radius slowest, so that a warp's tasks share r (the initial sum's trip count)
      for (int task = threadIdx.x; task < gn * nr * nseg; task += ST_NT) {
        const int sg = task % nseg;
        const int iq = task / nseg;
        const int i = iq % gn, q = iq / gn;
        const int r = A.radii[q];
        const float fn = A.fn[q], rn = A.rn[q];
        const float* vv = V + ((i * nr + q) * 2) * ST_ROW;
        const float* vw = vv + ST_ROW;
        float* mrow = M + (i * nr + q) * MROW;
        const int c0 = A.R + sg * ST_HSEG;
        CSum hv, hw;
        for (int k = c0 - r; k <= c0 + r; ++k) {
          hv.add(vv[sidx(k)]);
          if (nanw) hw.add(vw[sidx(k)]);
        }
        const int jn = min(ST_HSEG, TW - sg * ST_HSEG);
        for (int j = 0; j < jn; ++j) {
          const float num = div_by(hv.value(), fn, rn);
          float mean = num;
          if (nanw) {
            const float den = div_by(hw.value(), fn, rn);
            mean = den > 0.f ? __fdiv_rn(num, den) : 0.f;
          }
          mrow[midx(sg * ST_HSEG + j)] = mean;
          if (j + 1 < jn) {
            hv.add(vv[sidx(c0 + j + r + 1)]);
            hv.add(-vv[sidx(c0 + j - r)]);
            if (nanw) {
              hw.add(vw[sidx(c0 + j + r + 1)]);
              hw.add(-vw[sidx(c0 + j - r)]);
            }
          }
        }
      }
      __syncthreads();
      // (3) per pixel: radii in order, decimated radii, large field, scale, encoding
      for (int p = threadIdx.x; p < gn * TW; p += ST_NT) {
        const int i = p / TW, j = p - (p / TW) * TW;
        const int y = yg + i, x = I.x0 + j;
        if (x >= xend) continue;
        const float zv = z.at(y, x);
        float a = 0.f;
#pragma unroll
        for (int q = 0; q < NR; ++q) {
          const float d = __fmul_rn(A.weights[q], __fsub_rn(zv, M[(i * nr + q) * MROW + midx(j)]));
          a = q == 0 ? d : __fadd_rn(a, d);
        }
        for (int dd = 0; dd < T.ndec; ++dd) {
          const DecK& D = T.dec[dd];
          const int y0 = DYi[(dd * ST_G + i) * 2], y1 = DYi[(dd * ST_G + i) * 2 + 1];
          const int x0 = DXi[(dd * TW + j) * 2], x1 = DXi[(dd * TW + j) * 2 + 1];
          const float fy = DYf[dd * ST_G + i], fx = DXf[dd * TW + j];
          const float* m = D.ms;
          const float ma = __ldg(m + (long long)y0 * D.w + x0), mb = __ldg(m + (long long)y0 * D.w + x1);
          const float mc = __ldg(m + (long long)y1 * D.w + x0), md = __ldg(m + (long long)y1 * D.w + x1);
          const float top = fmaf(fx, mb - ma, ma), bot = fmaf(fx, md - mc, mc);
          const float mean = fmaf(fy, bot - top, top);
          const float t = __fmul_rn(D.weight, __fsub_rn(zv, mean));
          a = (nr == 0 && dd == 0) ? t : __fadd_rn(a, t);
        }
        float v;
        if (zv != zv) {
          v = kQNaN;
        } else {
          const bool have_large = A.field != nullptr;
          float large = 0.f;
          if (have_large) large = __fsub_rn(__fmul_rn(A.w_large, zv), field_at(A, T.gy0 + y, T.gx0 + x));
          if (A.have_small) v = have_large ? __fadd_rn(a, large) : a;
          else v = large;
          if (A.scale > 0.f) v = __fdiv_rn(v, A.scale);
        }
        const long long off = (long long)(y - T.cy0) * A.old + (x - T.cx0);
        if (A.dtype == FSG_F32) reinterpret_cast<float*>(T.out)[off] = v;
        else if (A.dtype == FSG_U8) reinterpret_cast<uint8_t*>(T.out)[off] = (uint8_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
        else reinterpret_cast<int16_t*>(T.out)[off] = (int16_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
      }
      __syncthreads();
    }
  }
}

// ------------------------------------ fused full-resolution pass, exact sums
// The same work as topousm_strip with every box sum computed exactly in 64-bit
// fixed point.  A cell contributes q = (rint(z * 2^k) << FX_CB) + valid (0 for
// NoData), so one integer sum carries both the value sum and the valid count
// of a box; the count stays below 2^FX_CB and the value part below 2^63, so
// the low FX_CB bits of any box sum are its count and the rest its value sum,
// even though the running sums themselves wrap modulo 2^64 (unsigned).  k is
// chosen per launch from max |z| over the windows.  The box mean is then
// sum * 2^-k / count, rounded once: the reference's separable float32 means
// (uniform_filter per axis, float32 intermediate; NaN-aware num/den) agree with
// it to within two float32 ulps, and no running sum drifts.
//
// Per strip of FX_NT buffer columns (window columns x0-R .. x0-R+255, 'reflect'
// at the window edges) and per row t of the window (rows 'reflect'ed too):
//   E[t][j] = sum_{b < j} q[t][b]                  (row prefix, j = 0..256)
// is kept in a ring of 2R+2G+1 rows in shared memory, so one row prefix serves
// every radius.  Thread c owns output column c (buffer column b = R + c) and
// keeps, per radius, the box sum of its pixel as a running sum over rows:
//   D_r(y) = sum_{t = y-r}^{y+r} (E[t][b+r+1] - E[t][b-r]).
// Rows go in groups of G: while the threads walk the group's rows (four ring
// reads per radius and row), each warp prefix-sums one row of the next group
// into the ring; one barrier per group.  The coarse-field and decimated-grid
// corner values a thread needs change only every few rows and stay in
// registers.
constexpr int FX_NT = 256, FX_CB = 15, FX_G = 8, FX_MAXNR = 4;
constexpr int FX_EP = 257 + 16;  // padded pitch of a 257-entry row: entry j at j + j / 16
__device__ __forceinline__ int fx_idx(int j) { return j + (j >> 4); }
typedef unsigned long long u64;

// max |z| over the valid cells of every window, as float bits (atomicMax on
// the bit pattern orders non-negative floats); blockIdx.y = tile.
__global__ void window_absmax(const TopoTileK* tiles, unsigned* zmax, int* nan_flags) {
  const TopoTileK& T = tiles[blockIdx.y];
  const ZView& z = T.z;
  float m[4] = {0.f, 0.f, 0.f, 0.f};
  bool dirty = false;  // NoData or a non-finite value seen (the window's flag in nan_flags)
  for (int y = blockIdx.x; y < z.h; y += gridDim.x) {
    const float* row = z.p + (long long)y * z.ld;
    // scalar head up to a 16-byte boundary, float4 body, scalar tail
    const int head = min(z.w, (int)((16 - ((uintptr_t)row & 15)) & 15) / 4);
    const int nv = (z.w - head) / 4;
    for (int x = threadIdx.x; x < head; x += blockDim.x) {
      const float v = __ldg(row + x);
      if (!is_nodata(v, z.ndf, z.has_nodata != 0)) m[0] = fmaxf(m[0], fabsf(v));
      dirty |= !isfinite(v) || is_nodata(v, z.ndf, z.has_nodata != 0);
    }
    if (((uintptr_t)row & 3) == 0) {
      const float4* r4 = reinterpret_cast<const float4*>(row + head);
      for (int k = threadIdx.x; k < nv; k += blockDim.x) {
        const float4 v = __ldg(r4 + k);
        const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (!is_nodata(e[q], z.ndf, z.has_nodata != 0)) m[q] = fmaxf(m[q], fabsf(e[q]));
          dirty |= !isfinite(e[q]) || is_nodata(e[q], z.ndf, z.has_nodata != 0);
        }
      }
    } else {
      for (int x = head + threadIdx.x; x < head + 4 * nv; x += blockDim.x) {
        const float v = __ldg(row + x);
        if (!is_nodata(v, z.ndf, z.has_nodata != 0)) m[1] = fmaxf(m[1], fabsf(v));
        dirty |= !isfinite(v) || is_nodata(v, z.ndf, z.has_nodata != 0);
      }
    }
    for (int x = head + 4 * nv + threadIdx.x; x < z.w; x += blockDim.x) {
      const float v = __ldg(row + x);
      if (!is_nodata(v, z.ndf, z.has_nodata != 0)) m[2] = fmaxf(m[2], fabsf(v));
      dirty |= !isfinite(v) || is_nodata(v, z.ndf, z.has_nodata != 0);
    }
  }
  if (__syncthreads_or(dirty) && threadIdx.x == 0) nan_flags[blockIdx.y] = 1;
  float mm = fmaxf(fmaxf(m[0], m[1]), fmaxf(m[2], m[3]));
  for (int o = 16; o > 0; o >>= 1) mm = fmaxf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
  __shared__ float wm[32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = mm;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) mm = fmaxf(mm, wm[w]);
    mm = fmaxf(mm, wm[0]);
    if (isfinite(mm)) atomicMax(zmax, __float_as_uint(mm));
  }
}

// Shared memory of topousm_fixed (bytes): the prefix ring, the per-group table
// of ring-row offsets (entering / leaving row of each radius) and the
// decimated grids' row coordinates of a group.
struct FxSmem {
  static size_t bytes(int ring) {
    return sizeof(u64) * FX_EP * (size_t)ring + sizeof(int2) * FX_G * FX_MAXNR + 3 * sizeof(float) * ST_MAXD * FX_G;
  }
};

template <int NR>
__global__ void __launch_bounds__(FX_NT, 1) topousm_fixed(const __grid_constant__ StripArgs A) {
  extern __shared__ __align__(16) u64 fsm[];
  constexpr int G = FX_G;
  constexpr int ROWB = FX_EP * 8;  // bytes per ring row
  const int RING = A.ring, TW = A.TW, R = A.R;
  u64* ring = fsm;
  int2* OFF = reinterpret_cast<int2*>(ring + (size_t)RING * FX_EP);  // [G][FX_MAXNR] byte offsets
  int* DYi = reinterpret_cast<int*>(OFF + G * FX_MAXNR);             // [ST_MAXD][G][2]
  float* DYf = reinterpret_cast<float*>(DYi + 2 * ST_MAXD * G);      // [ST_MAXD][G]
  const char* ringb = reinterpret_cast<const char*>(ring);
  __shared__ TopoTileK Ts;
  const TopoTileK& T = Ts;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // warps 0 .. ncons-1 own the strip's output columns; the others prefix-sum rows
  const int ncons = min(FX_NT / 32, (TW + 31) / 32);
  const int nprod = FX_NT / 32 - ncons;
  // fixed-point scale 2^k: |z| < 2^e for every valid z, and e + k = 33 keeps
  // every box's value sum below 2^(33 + log2(129^2) + FX_CB) < 2^63
  const unsigned mb = *A.zmax;
  const int e = mb ? (int)((mb >> 23) & 0xFF) - 126 : 0;
  const int k = max(-100, min(100, 33 - e));
  const float sk = ldexpf(1.0f, k), isk = ldexpf(1.0f, -k);
  // entry 0 of every prefix row is 0 and never written again
  for (int r = tid; r < RING; r += FX_NT) ring[(size_t)r * FX_EP] = 0ull;
  const int c = tid;               // output column of this thread within the strip
  const int b = R + c;             // its buffer column
  // per-radius constants: prefix-column byte offsets, weight, full box count and RN(1/count)
  int ja[NR], jb[NR], n2[NR];
  float wq[NR], n2f[NR], rn2[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    const int r = A.radii[q];
    ja[q] = c < TW ? fx_idx(b + r + 1) * 8 : 0;
    jb[q] = c < TW ? fx_idx(b - r) * 8 : 0;
    n2[q] = (2 * r + 1) * (2 * r + 1);
    n2f[q] = (float)n2[q];
    rn2[q] = 1.0f / n2f[q];
    wq[q] = A.weights[q];
  }
  const int nitems = A.nitems_dev ? *A.nitems_dev : A.nitems;  // device-built list: tensor-path fix-up
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const StripItem I = A.items[it];
    __syncthreads();
    for (int q = tid; q < (int)(sizeof(TopoTileK) / 4); q += FX_NT)
      reinterpret_cast<int*>(&Ts)[q] = reinterpret_cast<const int*>(A.tiles + I.tile)[q];
    __syncthreads();
    const ZView z = T.z;
    const int y0 = I.y0, y1 = I.y1, x0 = I.x0;
    const int xb = x0 - R;                          // window column of buffer column 0
    const int x = x0 + c;
    const bool active = c < TW && x < min(x0 + TW, T.cx0 + T.cw);
    const int tbase = y0 - R;                       // ring slot of row t: (t - tbase) % RING
    const bool vec = xb >= 0 && xb + FX_NT <= z.w && (z.ld & 3) == 0 &&
                     ((reinterpret_cast<uintptr_t>(z.p + xb) & 15) == 0);
    // one row of the window (reflected) -> this lane's 8 buffer columns 8*lane .. 8*lane+7
    auto load_row = [&](int t, float (&v)[8]) {
      const float* row = z.p + (long long)reflect_idx(t, z.h) * z.ld;
      if (vec) {
        const float4* p4 = reinterpret_cast<const float4*>(row + xb + 8 * lane);
        const float4 a4 = __ldg(p4), b4 = __ldg(p4 + 1);
        v[0] = a4.x; v[1] = a4.y; v[2] = a4.z; v[3] = a4.w;
        v[4] = b4.x; v[5] = b4.y; v[6] = b4.z; v[7] = b4.w;
      } else {
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = __ldg(row + reflect_idx(xb + 8 * lane + m, z.w));
      }
    };
    // fixed-point cells, warp-wide prefix, store E[t][1..256] into the ring
    auto scan_store = [&](int t, const float (&v)[8]) {
      u64 pm[8];
      u64 acc = 0ull;
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const float xv = v[m];
        const bool ok = !is_nodata(xv, z.ndf, z.has_nodata != 0);
        const u64 q = ok ? ((u64)__float2ll_rn(__fmul_rn(xv, sk)) << FX_CB) + 1ull : 0ull;
        acc += q;
        pm[m] = acc;
      }
      u64 incl = acc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u64 n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
      }
      const u64 excl = incl - acc;
      u64* row = ring + (size_t)((t - tbase) % RING) * FX_EP;
#pragma unroll
      for (int m = 0; m < 8; ++m) row[fx_idx(8 * lane + m + 1)] = excl + pm[m];
    };
    // prologue: rows tbase .. y0 + G + R - 1 (those the first group needs)
    {
      const int tend = min(y0 + G + R, y1 + R);
      for (int t = tbase + warp; t < tend; t += FX_NT / 32) {
        float v[8];
        load_row(t, v);
        scan_store(t, v);
      }
    }
    // column coordinates of the coarse field and of the decimated grids (fixed per item)
    const bool have_large = A.field != nullptr;
    int fxa = 0, fxb = 0;
    float ftx = 0.f;
    if (have_large) {
      const float cx = __fsub_rn(__fmul_rn(__fadd_rn((float)(T.gx0 + x), 0.5f), A.sx), 0.5f);
      const float f0 = floorf(cx);
      ftx = cx - f0;
      fxa = clamp_idx((int)f0, A.fw);
      fxb = clamp_idx((int)f0 + 1, A.fw);
    }
    int dxa[ST_MAXD], dxb[ST_MAXD], dya[ST_MAXD];
    float dfx[ST_MAXD], dm[ST_MAXD][4];
#pragma unroll
    for (int d = 0; d < ST_MAXD; ++d) {
      dxa[d] = dxb[d] = 0;
      dya[d] = -1;
      dfx[d] = 0.f;
      if (d < T.ndec) {
        const DecK& D = T.dec[d];
        const double cc = (double)x * D.zx;
        const int sx = (int)floor(cc);
        dxa[d] = clamp_idx(sx, D.w);
        dxb[d] = clamp_idx(sx + 1, D.w);
        dfx[d] = (float)(cc - (double)sx);
      }
      dm[d][0] = dm[d][1] = dm[d][2] = dm[d][3] = 0.f;
    }
    int fya = INT_MIN;
    float fa = 0.f, fb = 0.f, fc = 0.f, fd = 0.f;
    const float* zp = z.p + (long long)y0 * z.ld + x;   // this column, current row
    const size_t esz = A.dtype == FSG_F32 ? 4 : (A.dtype == FSG_I16 ? 2 : 1);
    char* op = T.out + ((long long)(y0 - T.cy0) * A.old + (x - T.cx0)) * (long long)esz;
    const long long ostep = A.old * (long long)esz;
    __syncthreads();
    // the box sums of row y0 (2r+1 rows of the ring per radius)
    u64 D[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      const int r = A.radii[q];
      u64 s = 0ull;
      if (active)
        for (int t = y0 - r; t <= y0 + r; ++t) {
          const char* row = ringb + (size_t)((t - tbase) % RING) * ROWB;
          s += *reinterpret_cast<const u64*>(row + ja[q]) - *reinterpret_cast<const u64*>(row + jb[q]);
        }
      D[q] = s;
    }
    float zn = active ? __ldg(zp) : 0.f;  // z of the next row (prefetched)
    for (int yg = y0; yg < y1; yg += G) {
      const int gn = min(G, y1 - yg);
      // ring-row byte offsets of the group: entering row y + r, leaving row y - 1 - r
      if (tid < G * NR) {
        const int i = tid / NR, q = tid - (tid / NR) * NR;
        const int r = A.radii[q];
        const int y = yg + i;
        int se = (y + r - tbase) % RING;
        int sl = y - 1 - r - tbase;
        sl = sl < 0 ? 0 : sl % RING;  // (row y0's sums are built directly)
        OFF[i * FX_MAXNR + q] = make_int2(se * ROWB, sl * ROWB);
      } else if (tid >= 64 && tid < 64 + T.ndec * G) {  // decimated-grid row coordinates
        const int d = (tid - 64) / G, i = (tid - 64) - ((tid - 64) / G) * G;
        const DecK& Dk = T.dec[d];
        const double cc = (double)(yg + i) * Dk.zy;
        const int sy2 = (int)floor(cc);
        DYi[(d * G + i) * 2] = clamp_idx(sy2, Dk.h);
        DYi[(d * G + i) * 2 + 1] = clamp_idx(sy2 + 1, Dk.h);
        DYf[d * G + i] = (float)(cc - (double)sy2);
      }
      const bool more = yg + G < y1;  // a next group exists: its rows go into the ring now
      float nv[8];
      const int tn1 = yg + G + R + warp;
      const bool scan1 = nprod == 0 && more && tn1 < y1 + R;
      if (scan1) load_row(tn1, nv);
      __syncthreads();  // tables
      if (warp < ncons && active) {
#pragma unroll 2
        for (int i = 0; i < gn; ++i) {
          const int y = yg + i;
          const float zv = zn;
          if (y + 1 < y1) zn = __ldg(zp + z.ld);
          zp += z.ld;
          float a = 0.f;
#pragma unroll
          for (int q = 0; q < NR; ++q) {
            if (y > y0) {
              const int2 o = OFF[i * FX_MAXNR + q];
              const u64 ea = *reinterpret_cast<const u64*>(ringb + o.x + ja[q]);
              const u64 eb = *reinterpret_cast<const u64*>(ringb + o.x + jb[q]);
              const u64 la = *reinterpret_cast<const u64*>(ringb + o.y + ja[q]);
              const u64 lb = *reinterpret_cast<const u64*>(ringb + o.y + jb[q]);
              D[q] += (ea - eb) - (la - lb);
            }
            const long long S = (long long)D[q];
            const int cnt = (int)S & ((1 << FX_CB) - 1);
            const float num = __fmul_rn(__ll2float_rn(S >> FX_CB), isk);
            float mean;
            if (cnt == n2[q]) {  // no NoData in the box: divide by the fixed count (Markstein)
              const float qq = __fmul_rn(num, rn2[q]);
              mean = __fmaf_rn(__fmaf_rn(-qq, n2f[q], num), rn2[q], qq);
            } else if (cnt > 0) {
              const float dn = (float)cnt, rr = rcp_approx(dn);
              const float qq = __fmul_rn(num, rr);
              mean = __fmaf_rn(__fmaf_rn(-qq, dn, num), rr, qq);
            } else {
              mean = 0.f;
            }
            const float dq = __fmul_rn(wq[q], __fsub_rn(zv, mean));
            a = q == 0 ? dq : __fadd_rn(a, dq);
          }
#pragma unroll
          for (int dd = 0; dd < ST_MAXD; ++dd) {
            if (dd >= T.ndec) break;
            const DecK& Dk = T.dec[dd];
            const int ya = DYi[(dd * G + i) * 2];
            if (ya != dya[dd]) {  // new decimated row pair (uniform across the block)
              const int yb = DYi[(dd * G + i) * 2 + 1];
              const float* m = Dk.ms;
              dm[dd][0] = __ldg(m + (long long)ya * Dk.w + dxa[dd]);
              dm[dd][1] = __ldg(m + (long long)ya * Dk.w + dxb[dd]);
              dm[dd][2] = __ldg(m + (long long)yb * Dk.w + dxa[dd]);
              dm[dd][3] = __ldg(m + (long long)yb * Dk.w + dxb[dd]);
              dya[dd] = ya;
            }
            const float fy = DYf[dd * G + i], fx = dfx[dd];
            const float top = fmaf(fx, dm[dd][1] - dm[dd][0], dm[dd][0]);
            const float bot = fmaf(fx, dm[dd][3] - dm[dd][2], dm[dd][2]);
            const float mean = fmaf(fy, bot - top, top);
            const float t = __fmul_rn(Dk.weight, __fsub_rn(zv, mean));
            a = (NR == 0 && dd == 0) ? t : __fadd_rn(a, t);
          }
          const bool nan = is_nodata(zv, z.ndf, z.has_nodata != 0);
          float v;
          if (nan) {
            v = kQNaN;
          } else {
            float large = 0.f;
            if (have_large) {
              // _nan_utils.py:276-281 (as field_at), with the column part fixed per item
              const float cy = __fsub_rn(__fmul_rn(__fadd_rn((float)(T.gy0 + y), 0.5f), A.sy), 0.5f);
              const float f0 = floorf(cy);
              const float ty = cy - f0;
              if ((int)f0 != fya) {  // keyed on the unclamped row: both rows clamp at the top edge
                const int ya = clamp_idx((int)f0, A.fh), yb = clamp_idx((int)f0 + 1, A.fh);
                const float* F = A.field;
                fa = __ldg(F + ya * A.fld + fxa);
                fb = __ldg(F + ya * A.fld + fxb);
                fc = __ldg(F + yb * A.fld + fxa);
                fd = __ldg(F + yb * A.fld + fxb);
                fya = (int)f0;
              }
              const float top = fmaf(ftx, fb - fa, fa);
              const float bot = fmaf(ftx, fd - fc, fc);
              large = __fsub_rn(__fmul_rn(A.w_large, zv), fmaf(ty, bot - top, top));
            }
            if (A.have_small) v = have_large ? __fadd_rn(a, large) : a;
            else v = large;
            if (A.scale > 0.f) v = div_by(v, A.scale, A.rscale);
          }
          if (A.dtype == FSG_F32) *reinterpret_cast<float*>(op) = v;
          else if (A.dtype == FSG_U8) *reinterpret_cast<uint8_t*>(op) = (uint8_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
          else *reinterpret_cast<int16_t*>(op) = (int16_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
          op += ostep;
        }
      } else if (warp >= ncons && more) {
        // producer warps: the next group's rows into the ring
        for (int tn = yg + G + R + (warp - ncons); tn < min(yg + 2 * G + R, y1 + R); tn += nprod) {
          float v[8];
          load_row(tn, v);
          scan_store(tn, v);
        }
      }
      if (scan1) scan_store(tn1, nv);
      __syncthreads();  // ring rows of the next group; tables free
    }
  }
}

// Hybrid variant for two or more full-resolution radii: the prefix ring holds
// only the rows of the smaller radii (2 Rs + G + 1 rows, Rs = the second
// largest radius), and the largest radius R takes, per group of G rows, its
// entering rows y+R and leaving rows y-1-R from two G-row buffers that the warps
// prefix-sum for that group (those rows are read again from L2).  With the
// default radii (2, 8, 32) a CTA needs ~90 KB instead of 178 KB, so two CTAs
// share an SM.  Each group runs a scan phase (all warps: the group's new ring
// rows and its entering / leaving rows of R) and a pixel phase (output-column
// warps), with a barrier after each; the other CTA of the SM fills the gaps.
// The running sum of R for the first row of an item is built by adding its
// 2R+1 rows through the entering buffer, G rows at a time.
constexpr int HY_MAXNR = FX_MAXNR;
struct HySmem {
  static size_t bytes(int ring, int G) {
    return sizeof(u64) * FX_EP * ((size_t)ring + 2 * G) + sizeof(int2) * G * HY_MAXNR +
           3 * sizeof(float) * ST_MAXD * G;
  }
};

// HNT threads (>= the strip's output columns), G rows per group, MINB CTAs per SM.
// CLEAN: the items of windows without NoData (partition_items sorts them out with the
// windows' flags from the pass that took their max |z|): the cells carry no valid-count
// bits and every box holds (2r+1)^2 cells -- the same sums and means as the general
// kernel, with fewer instructions.
template <int NR, int HNT, int G, int MINB, bool CLEAN>
__global__ void __launch_bounds__(HNT, MINB) topousm_hybrid(const __grid_constant__ StripArgs A) {
  static_assert(NR >= 2, "the hybrid kernel needs a ring radius and a large radius");
  extern __shared__ __align__(16) u64 fsm[];
  constexpr int NS = NR - 1;  // radii served by the ring
  const int RING = A.ring, TW = A.TW, R = A.R;
  u64* ring = fsm;
  u64* BE = ring + (size_t)RING * FX_EP;                     // [G][FX_EP] entering rows of R
  u64* BL = BE + (size_t)G * FX_EP;                          // [G][FX_EP] leaving rows of R
  int2* OFF = reinterpret_cast<int2*>(BL + (size_t)G * FX_EP);  // [G][HY_MAXNR] ring-row element offsets
  int* DYi = reinterpret_cast<int*>(OFF + G * HY_MAXNR);     // [ST_MAXD][G][2]
  float* DYf = reinterpret_cast<float*>(DYi + 2 * ST_MAXD * G);
  __shared__ TopoTileK Ts;
  const TopoTileK& T = Ts;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = HNT / 32;
  const int ncons = min(NW, (TW + 31) / 32);
  const unsigned mb = *A.zmax;
  const int e = mb ? (int)((mb >> 23) & 0xFF) - 126 : 0;
  const int k = max(-100, min(100, 33 - e));
  const float sk = ldexpf(1.0f, k), isk = ldexpf(1.0f, -k);
  for (int r = tid; r < RING; r += HNT) ring[(size_t)r * FX_EP] = 0ull;
  for (int r = tid; r < 2 * G; r += HNT) BE[(size_t)r * FX_EP] = 0ull;
  const int c = tid, b = R + c;
  int ja[NR], jb[NR];
  float wq[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    const int r = A.radii[q];
    ja[q] = c < TW ? fx_idx(b + r + 1) : 0;
    jb[q] = c < TW ? fx_idx(b - r) : 0;
    wq[q] = A.weights[q];
  }
  const int Rs = A.radii[NS - 1];
  const int nitems = A.nitems_dev ? *A.nitems_dev : A.nitems;  // device-built list: tensor-path fix-up
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const StripItem I = A.items[it];
    __syncthreads();
    for (int q = tid; q < (int)(sizeof(TopoTileK) / 4); q += HNT)
      reinterpret_cast<int*>(&Ts)[q] = reinterpret_cast<const int*>(A.tiles + I.tile)[q];
    __syncthreads();
    const ZView z = T.z;
    const int y0 = I.y0, y1 = I.y1, x0 = I.x0;
    const int xb = x0 - R;
    const int x = x0 + c;
    const bool active = c < TW && x < min(x0 + TW, T.cx0 + T.cw);
    const int tbase = y0 - Rs;  // ring slot of row t: (t - tbase) % RING
    const bool vec = xb >= 0 && xb + FX_NT <= z.w && (z.ld & 3) == 0 &&
                     ((reinterpret_cast<uintptr_t>(z.p + xb) & 15) == 0);
    // row t of the window (reflected) -> prefix sums E[t][1..256] at dst
    auto scan_row = [&](int t, u64* dst) {
      float v[8];
      const float* row = z.p + (long long)reflect_idx(t, z.h) * z.ld;
      if (vec) {
        const float4* p4 = reinterpret_cast<const float4*>(row + xb + 8 * lane);
        const float4 a4 = __ldg(p4), b4 = __ldg(p4 + 1);
        v[0] = a4.x; v[1] = a4.y; v[2] = a4.z; v[3] = a4.w;
        v[4] = b4.x; v[5] = b4.y; v[6] = b4.z; v[7] = b4.w;
      } else {
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = __ldg(row + reflect_idx(xb + 8 * lane + m, z.w));
      }
      u64 pm[8];
      u64 acc = 0ull;
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const float xv = v[m];
        u64 q;
        if constexpr (CLEAN) {
          q = (u64)__float2ll_rn(__fmul_rn(xv, sk));
        } else {
          const bool ok = !is_nodata(xv, z.ndf, z.has_nodata != 0);
          q = ok ? ((u64)__float2ll_rn(__fmul_rn(xv, sk)) << FX_CB) + 1ull : 0ull;
        }
        acc += q;
        pm[m] = acc;
      }
      u64 incl = acc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u64 n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
      }
      const u64 excl = incl - acc;
#pragma unroll
      for (int m = 0; m < 8; ++m) dst[fx_idx(8 * lane + m + 1)] = excl + pm[m];
    };
    auto ring_row = [&](int t) { return ring + (size_t)((t - tbase) % RING) * FX_EP; };
    // prologue: ring rows y0-Rs .. y0+Rs
    for (int t = tbase + warp; t <= y0 + Rs; t += NW) scan_row(t, ring_row(t));
    // columns of the coarse field and of the decimated grids (fixed per item)
    const bool have_large = A.field != nullptr;
    int fxa = 0, fxb = 0;
    float ftx = 0.f;
    if (have_large) {
      const float cx = __fsub_rn(__fmul_rn(__fadd_rn((float)(T.gx0 + x), 0.5f), A.sx), 0.5f);
      const float f0 = floorf(cx);
      ftx = cx - f0;
      fxa = clamp_idx((int)f0, A.fw);
      fxb = clamp_idx((int)f0 + 1, A.fw);
    }
    int dxa[ST_MAXD], dxb[ST_MAXD], dya[ST_MAXD];
    float dfx[ST_MAXD], dm[ST_MAXD][4];
#pragma unroll
    for (int d = 0; d < ST_MAXD; ++d) {
      dxa[d] = dxb[d] = 0;
      dya[d] = -1;
      dfx[d] = 0.f;
      if (d < T.ndec) {
        const DecK& D = T.dec[d];
        const double cc = (double)x * D.zx;
        const int sx = (int)floor(cc);
        dxa[d] = clamp_idx(sx, D.w);
        dxb[d] = clamp_idx(sx + 1, D.w);
        dfx[d] = (float)(cc - (double)sx);
      }
      dm[d][0] = dm[d][1] = dm[d][2] = dm[d][3] = 0.f;
    }
    int fya = INT_MIN;
    float fa = 0.f, fb = 0.f, fc = 0.f, fd = 0.f;
    const float* zp = z.p + (long long)y0 * z.ld + x;
    const size_t esz = A.dtype == FSG_F32 ? 4 : (A.dtype == FSG_I16 ? 2 : 1);
    char* op = T.out + ((long long)(y0 - T.cy0) * A.old + (x - T.cx0)) * (long long)esz;
    const long long ostep = A.old * (long long)esz;
    __syncthreads();
    // running sums of row y0: ring radii from the ring, R by adding its 2R+1 rows G at a time
    u64 D[NR];
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      const int r = A.radii[q];
      u64 s = 0ull;
      if (active)
        for (int t = y0 - r; t <= y0 + r; ++t) {
          const u64* row = ring_row(t);
          s += row[ja[q]] - row[jb[q]];
        }
      D[q] = s;
    }
    D[NS] = 0ull;
    for (int t0 = y0 - R; t0 <= y0 + R; t0 += G) {
      const int tn = min(G, y0 + R + 1 - t0);
      for (int i = warp; i < tn; i += NW) scan_row(t0 + i, BE + (size_t)i * FX_EP);
      __syncthreads();
      if (active)
        for (int i = 0; i < tn; ++i) D[NS] += BE[(size_t)i * FX_EP + ja[NS]] - BE[(size_t)i * FX_EP + jb[NS]];
      __syncthreads();
    }
    float zn = active ? __ldg(zp) : 0.f;  // z of the next row (prefetched)
    int tring = y0 + Rs;                  // last ring row scanned
    for (int yg = y0; yg < y1; yg += G) {
      const int gn = min(G, y1 - yg);
      // (scan phase) the group's new ring rows, its entering / leaving rows of R; tables
      {
        const int tr_end = min(yg + gn - 1 + Rs, y1 - 1 + Rs);
        const int nring = max(0, tr_end - tring);
        const int jobs = nring + 2 * gn;
        for (int jdx = warp; jdx < jobs; jdx += NW) {
          if (jdx < nring) {
            const int t = tring + 1 + jdx;
            scan_row(t, ring_row(t));
          } else {
            const int i = (jdx - nring) % gn, leave = (jdx - nring) / gn;
            const int y = yg + i;
            if (y > y0) scan_row(leave ? y - 1 - R : y + R, (leave ? BL : BE) + (size_t)i * FX_EP);
          }
        }
        tring = max(tring, tr_end);
        if (tid < G * NS) {
          const int i = tid / NS, q = tid - (tid / NS) * NS;
          const int r = A.radii[q];
          const int y = yg + i;
          const int se = (y + r - tbase) % RING;
          int sl = y - 1 - r - tbase;
          sl = sl < 0 ? 0 : sl % RING;
          OFF[i * HY_MAXNR + q] = make_int2(se * FX_EP, sl * FX_EP);
        } else if (tid >= 32 && tid < 32 + T.ndec * G) {
          const int d = (tid - 32) / G, i = (tid - 32) - ((tid - 32) / G) * G;
          const DecK& Dk = T.dec[d];
          const double cc = (double)(yg + i) * Dk.zy;
          const int sy2 = (int)floor(cc);
          DYi[(d * G + i) * 2] = clamp_idx(sy2, Dk.h);
          DYi[(d * G + i) * 2 + 1] = clamp_idx(sy2 + 1, Dk.h);
          DYf[d * G + i] = (float)(cc - (double)sy2);
        }
      }
      __syncthreads();
      // (pixel phase)
      if (warp < ncons && active) {
        for (int i = 0; i < gn; ++i) {
          const int y = yg + i;
          const float zv = zn;
          if (y + 1 < y1) zn = __ldg(zp + z.ld);
          zp += z.ld;
          float a = 0.f;
#pragma unroll
          for (int q = 0; q < NR; ++q) {
            if (y > y0) {
              if (q < NS) {
                const int2 o = OFF[i * HY_MAXNR + q];
                D[q] += (fsm[o.x + ja[q]] - fsm[o.x + jb[q]]) - (fsm[o.y + ja[q]] - fsm[o.y + jb[q]]);
              } else {
                const u64* be = BE + (size_t)i * FX_EP;
                const u64* bl = BL + (size_t)i * FX_EP;
                D[q] += (be[ja[q]] - be[jb[q]]) - (bl[ja[q]] - bl[jb[q]]);
              }
            }
            const long long S = (long long)D[q];
            float mean;
            if constexpr (CLEAN) {  // S is the value sum, the count (2r+1)^2 ('reflect' keeps boxes full)
              const float num = __fmul_rn(__ll2float_rn(S), isk);
              const float dn = __fmul_rn(A.fn[q], A.fn[q]), rr = rcp_approx(dn);
              const float qq = __fmul_rn(num, rr);
              mean = __fmaf_rn(__fmaf_rn(-qq, dn, num), rr, qq);
            } else {
              const int cnt = (int)S & ((1 << FX_CB) - 1);
              const float num = __fmul_rn(__ll2float_rn(S >> FX_CB), isk);
              const float dn = (float)max(cnt, 1), rr = rcp_approx(dn);  // Markstein-corrected num / cnt
              const float qq = __fmul_rn(num, rr);
              mean = cnt > 0 ? __fmaf_rn(__fmaf_rn(-qq, dn, num), rr, qq) : 0.f;
            }
            const float dq = __fmul_rn(wq[q], __fsub_rn(zv, mean));
            a = q == 0 ? dq : __fadd_rn(a, dq);
          }
#pragma unroll
          for (int dd = 0; dd < ST_MAXD; ++dd) {
            if (dd >= T.ndec) break;
            const DecK& Dk = T.dec[dd];
            const int ya = DYi[(dd * G + i) * 2];
            if (ya != dya[dd]) {
              const int yb = DYi[(dd * G + i) * 2 + 1];
              const float* m = Dk.ms;
              dm[dd][0] = __ldg(m + (long long)ya * Dk.w + dxa[dd]);
              dm[dd][1] = __ldg(m + (long long)ya * Dk.w + dxb[dd]);
              dm[dd][2] = __ldg(m + (long long)yb * Dk.w + dxa[dd]);
              dm[dd][3] = __ldg(m + (long long)yb * Dk.w + dxb[dd]);
              dya[dd] = ya;
            }
            const float fy = DYf[dd * G + i], fx = dfx[dd];
            const float top = fmaf(fx, dm[dd][1] - dm[dd][0], dm[dd][0]);
            const float bot = fmaf(fx, dm[dd][3] - dm[dd][2], dm[dd][2]);
            const float mean = fmaf(fy, bot - top, top);
            a = __fadd_rn(a, __fmul_rn(Dk.weight, __fsub_rn(zv, mean)));
          }
          float v;
          if (!CLEAN && is_nodata(zv, z.ndf, z.has_nodata != 0)) {
            v = kQNaN;
          } else {
            float large = 0.f;
            if (have_large) {
              const float cy = __fsub_rn(__fmul_rn(__fadd_rn((float)(T.gy0 + y), 0.5f), A.sy), 0.5f);
              const float f0 = floorf(cy);
              const float ty = cy - f0;
              if ((int)f0 != fya) {
                const int ya = clamp_idx((int)f0, A.fh), yb = clamp_idx((int)f0 + 1, A.fh);
                const float* F = A.field;
                fa = __ldg(F + ya * A.fld + fxa);
                fb = __ldg(F + ya * A.fld + fxb);
                fc = __ldg(F + yb * A.fld + fxa);
                fd = __ldg(F + yb * A.fld + fxb);
                fya = (int)f0;
              }
              const float top = fmaf(ftx, fb - fa, fa);
              const float bot = fmaf(ftx, fd - fc, fc);
              large = __fsub_rn(__fmul_rn(A.w_large, zv), fmaf(ty, bot - top, top));
            }
            v = have_large ? __fadd_rn(a, large) : a;
            if (A.scale > 0.f) v = div_by(v, A.scale, A.rscale);
          }
          if (A.dtype == FSG_F32) *reinterpret_cast<float*>(op) = v;
          else if (A.dtype == FSG_U8) *reinterpret_cast<uint8_t*>(op) = (uint8_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
          else *reinterpret_cast<int16_t*>(op) = (int16_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
          op += ostep;
        }
      }
      __syncthreads();
    }
  }
}

// The strip items split by their window's NoData flag: items of windows without
// NoData to `clean`, the others to `dirty` (counts zeroed before the launch; the
// order within a list does not matter: every item writes its own pixels).
__global__ void partition_items(const StripItem* items, int n, const TopoTileK* tiles, StripItem* clean,
                                int* nclean, StripItem* dirty, int* ndirty) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const StripItem it = items[i];
  if (*tiles[it.tile].nan_flag == 0) clean[atomicAdd(nclean, 1)] = it;
  else dirty[atomicAdd(ndirty, 1)] = it;
}

// flag[t] = any NoData in window t (ZView per tile); blockIdx.y = tile.
__global__ void window_nan_flags(const TopoTileK* tiles, int* flags) {
  const TopoTileK& T = tiles[blockIdx.y];
  const ZView& z = T.z;
  bool n = false;
  for (int y = blockIdx.x; y < z.h; y += gridDim.x)
    for (int x = threadIdx.x; x < z.w; x += blockDim.x) {
      const float v = z.at(y, x);
      n |= v != v;
    }
  if (__syncthreads_or(n) && threadIdx.x == 0) atomicOr(flags + blockIdx.y, 1);
}

// ------------------------------------------------------------------- host
struct Grid2 {
  dim3 g, b;
};

Grid2 grid2d(int h, int w) {
  Grid2 r;
  r.b = dim3(32, 8);
  r.g = dim3((w + 31) / 32, (h + 7) / 8);
  return r;
}

std::vector<float> gaussian_weights(double sigma, int* radius) {
  // scipy.ndimage._gaussian_kernel1d(sigma, 0, int(4*sigma + 0.5)), normalised in double.
  int R = (int)(4.0 * sigma + 0.5);
  std::vector<double> phi(2 * R + 1);
  double s = 0;
  for (int k = -R; k <= R; ++k) {
    phi[k + R] = std::exp(-0.5 / (sigma * sigma) * (double)k * (double)k);
    s += phi[k + R];
  }
  std::vector<float> g(R + 1);
  for (int k = 0; k <= R; ++k) g[k] = (float)(phi[k + R] / s);
  *radius = R;
  return g;
}

}  // namespace

// Filter engine with scratch; used by fsg_topousm, the coarse field and smoothing.
struct FilterCtx {
  cudaStream_t s;
  // Gaussian weight tables (device) for sigma = 1 and for the current void fill.
  float* g1 = nullptr;
  int r1 = 4;
};

static int upload(float* dst, const std::vector<float>& v, cudaStream_t s) {
  FSG_UPLOAD(dst, v.data(), v.size() * sizeof(float), s);
  return FSG_OK;
}

// Row-pass launch geometry: th rows x tw cols per block, shared-memory bounded.
static void row_geometry(int r, int nan_aware, int w, int* th, int* tw, size_t* smem) {
  static const int THS[] = {8, 4, 2, 1};
  for (int t : THS) {
    int ttw = NT * SEG / t;
    size_t bytes = (size_t)t * rp_pitch(ttw + 2 * r) * sizeof(float) * (nan_aware ? 2 : 1);
    if (bytes <= 96 * 1024 || t == 1) {
      *th = t;
      *tw = ttw;
      *smem = bytes;
      return;
    }
  }
}

template <class Src>
static int launch_box(const Src& src, int r, int nan_aware, AView vm, AView wm, RowArgs ra, cudaStream_t s) {
  const int chunk = 128;  // rows per block: (2r+1)/128 extra adds per row buys enough blocks for large r
  dim3 g((src.w + NT - 1) / NT, (src.h + chunk - 1) / chunk);
  box_cols<Src><<<g, NT, 0, s>>>(src, r, chunk, nan_aware, vm, wm);
  FSG_LAUNCHED(1);
  ra.vm = vm;
  ra.wm = wm;
  ra.r = r;
  ra.nan_aware = nan_aware;
  ra.gauss = 0;
  int th, tw;
  size_t smem;
  row_geometry(r, nan_aware, src.w, &th, &tw, &smem);
  ra.th = th;
  ra.tw = tw;
  if (smem > 48 * 1024) FSG_CUDA(cudaFuncSetAttribute(row_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 g2((src.w + tw - 1) / tw, (src.h + th - 1) / th);
  if (g2.y > 65535) return fail(FSG_ERR_UNSUPPORTED, "window of %d rows too tall for radius %d", src.h, r);
  row_pass<<<g2, NT, smem, s>>>(ra);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

template <class Src>
static int launch_gauss(const Src& src, const float* g, int R, int nan_aware, AView vm, AView wm, RowArgs ra,
                        cudaStream_t s) {
  dim3 gg((src.w + NT - 1) / NT, std::min(src.h, 65535));
  gauss_cols<Src><<<gg, NT, 0, s>>>(src, g, R, nan_aware, vm, wm, ra.run_if);
  FSG_LAUNCHED(1);
  ra.vm = vm;
  ra.wm = wm;
  ra.r = R;
  ra.nan_aware = nan_aware;
  ra.gauss = 1;
  ra.g = g;
  int th, tw;
  size_t smem;
  row_geometry(R, nan_aware, src.w, &th, &tw, &smem);
  ra.th = th;
  ra.tw = tw;
  if (smem > 48 * 1024) FSG_CUDA(cudaFuncSetAttribute(row_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 g2((src.w + tw - 1) / tw, (src.h + th - 1) / th);
  row_pass<<<g2, NT, smem, s>>>(ra);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

// _nan_utils.py:555-601 for algorithm 'topousm_fast' (algo factor 1.15).
int topousm_downsample_factor(double radius, double pixel_size) {
  double r = std::max(1.0, radius);
  double px = std::max(1e-3, pixel_size != 0.0 ? pixel_size : 1.0);
  double score = (r / 24.0) * 1.15 * 1.0 * std::pow(std::max(1.0, 1.0 / px), 0.35);
  if (score <= 1.0) return 1;
  double f = std::pow(2.0, std::floor(std::log2(score)));
  return (int)std::max(1.0, std::min(f, 16.0));
}

// Scratch for one window of at most h x w pixels.
struct TopoScratch {
  AView acc, vm, wm;       // h x w
  AView small, svm, swm, smean, ssv, ssw;  // (h/2+1) x (w/2+1)
  int* flag;
  float* g1;               // sigma = 1 weights (5 floats)
  float* gv;               // void-fill weights (<= 4097 floats)
  static size_t bytes(int h, int w) {
    size_t full = (size_t)h * w, sm = (size_t)((h + 1) / 2) * ((w + 1) / 2);
    return (3 * full + 6 * sm) * sizeof(float) + 256 + 8 * 1024 + 16 * 1024 + 6 * 256;
  }
  // decimation pipeline only (no full-size buffers)
  static size_t bytes_small(int h, int w) {
    size_t sm = (size_t)((h + 1) / 2) * ((w + 1) / 2);
    return 6 * ((sm * sizeof(float) + 255) & ~(size_t)255) + 256 + 8 * 1024 + 16 * 1024 + 6 * 256;
  }
  void carve_small(void* base, int h, int w) {
    char* p = static_cast<char*>(base);
    auto take = [&](size_t n) {
      char* q = p;
      p += (n + 255) & ~(size_t)255;
      return q;
    };
    int hs = (h + 1) / 2, ws = (w + 1) / 2;
    size_t sm = (size_t)hs * ws;
    acc = vm = wm = AView{nullptr, 0, 0, 0};
    AView* smalls[] = {&small, &svm, &swm, &smean, &ssv, &ssw};
    for (AView* a : smalls) *a = {reinterpret_cast<float*>(take(sm * 4)), ws, hs, ws};
    flag = reinterpret_cast<int*>(take(256));
    g1 = reinterpret_cast<float*>(take(8 * 1024));
    gv = reinterpret_cast<float*>(take(16 * 1024));
  }
  void carve(void* base, int h, int w) {
    char* p = static_cast<char*>(base);
    auto take = [&](size_t n) {
      char* q = p;
      p += (n + 255) & ~(size_t)255;
      return q;
    };
    size_t full = (size_t)h * w;
    int hs = (h + 1) / 2, ws = (w + 1) / 2;
    size_t sm = (size_t)hs * ws;
    acc = {reinterpret_cast<float*>(take(full * 4)), w, h, w};
    vm = {reinterpret_cast<float*>(take(full * 4)), w, h, w};
    wm = {reinterpret_cast<float*>(take(full * 4)), w, h, w};
    AView* smalls[] = {&small, &svm, &swm, &smean, &ssv, &ssw};
    for (AView* a : smalls) *a = {reinterpret_cast<float*>(take(sm * 4)), ws, hs, ws};
    flag = reinterpret_cast<int*>(take(256));
    g1 = reinterpret_cast<float*>(take(8 * 1024));
    gv = reinterpret_cast<float*>(take(16 * 1024));
  }
};

static AView resize(AView a, int h, int w) {
  a.h = h;
  a.w = w;
  a.ld = w;
  return a;
}

// Mean of `src` (an h x w view) for one radius at its own resolution, written
// into `out` (ROW_MEAN) -- used for decimated grids and the coarse field.
template <class Src>
static int mean_for_radius(const Src& src, int rr, TopoScratch& S, AView out, cudaStream_t s) {
  RowArgs ra;
  std::memset(&ra, 0, sizeof(ra));
  ra.mode = ROW_MEAN;
  ra.out = out;
  AView vm = resize(S.svm, src.h, src.w), wm = resize(S.swm, src.h, src.w);
  if (rr <= 1) return launch_gauss(src, S.g1, 4, 1, vm, wm, ra, s);
  return launch_box(src, rr, 1, vm, wm, ra, s);
}

// One window of topousm_fast: accumulates sum_r w_r (z - mean_r) into S.acc.
static int topousm_window(const ZView& z, const std::vector<int>& radii, const std::vector<float>& weights,
                          double pixel_size, TopoScratch& S, cudaStream_t s) {
  for (size_t i = 0; i < radii.size(); ++i) {
    const int r = radii[i];
    const float w = weights[i];
    const int first = i == 0;
    const int f = topousm_downsample_factor((double)r, pixel_size);
    if (f > 1) {
      const int hs = std::max(1, (z.h + f - 1) / f), ws = std::max(1, (z.w + f - 1) / f);
      AView small = resize(S.small, hs, ws);
      FSG_CUDA(cudaMemsetAsync(S.flag, 0, sizeof(int), s));
      Grid2 gd = grid2d(hs, ws);
      downsample_kernel<<<gd.g, gd.b, 0, s>>>(z, f, small, S.flag);
      FSG_LAUNCHED(1);
      // enclosed-void fill (runs only if the decimated grid holds NaN)
      double sigma = std::max(1.0, (double)std::min(hs, ws) / 64.0);
      int R;
      std::vector<float> gw = gaussian_weights(sigma, &R);
      if (R + 1 > 4096) return fail(FSG_ERR_UNSUPPORTED, "void-fill Gaussian radius %d too large", R);
      int st = upload(S.gv, gw, s);
      if (st) return st;
      {
        RowArgs ra;
        std::memset(&ra, 0, sizeof(ra));
        ra.mode = ROW_PAIR;
        ra.out = resize(S.ssv, hs, ws);
        ra.out2 = resize(S.ssw, hs, ws);
        ra.run_if = S.flag;
        st = launch_gauss(small, S.gv, R, 1, resize(S.svm, hs, ws), resize(S.swm, hs, ws), ra, s);
        if (st) return st;
        voidfill_combine<<<gd.g, gd.b, 0, s>>>(small, resize(S.ssv, hs, ws), resize(S.ssw, hs, ws), S.flag);
        FSG_LAUNCHED(1);
      }
      const int rs = std::max(1, (int)std::nearbyint((double)r / f));
      AView ms = resize(S.smean, hs, ws);
      st = mean_for_radius(small, rs, S, ms, s);
      if (st) return st;
      double zy = z.h > 1 ? (double)(hs - 1) / (double)(z.h - 1) : 1.0;
      double zx = z.w > 1 ? (double)(ws - 1) / (double)(z.w - 1) : 1.0;
      dim3 g((z.w + 31) / 32, (z.h + 31) / 32);
      accum_upsample<<<g, dim3(32, 8), 0, s>>>(z, ms, zy, zx, w, first, S.acc);
      FSG_LAUNCHED(1);
    } else {
      RowArgs ra;
      std::memset(&ra, 0, sizeof(ra));
      ra.mode = ROW_ACCUM;
      ra.out = S.acc;
      ra.z = z;
      ra.weight = w;
      ra.first = first;
      int st = r <= 1 ? launch_gauss(z, S.g1, 4, 1, S.vm, S.wm, ra, s) : launch_box(z, r, 1, S.vm, S.wm, ra, s);
      if (st) return st;
    }
  }
  return FSG_OK;
}

int prepare_g1(TopoScratch& S, cudaStream_t s) {
  int R;
  std::vector<float> g = gaussian_weights(1.0, &R);
  return upload(S.g1, g, s);
}

// The fused strip path applies when the radii ascend, the factor-1 radii come
// first (each 2..ST_MAXR, at most ST_MAXN of them) and at most ST_MAXD radii
// are decimated.
static bool strip_path_ok(const std::vector<int>& radii, double pixel_size, int* nfull) {
  int nf = 0, nd = 0;
  for (size_t i = 0; i < radii.size(); ++i) {
    if (i > 0 && radii[i] < radii[i - 1]) return false;
    if (topousm_downsample_factor((double)radii[i], pixel_size) == 1) {
      if (nd > 0 || radii[i] < 2 || radii[i] > ST_MAXR) return false;
      ++nf;
    } else {
      ++nd;
    }
  }
  if (nf > ST_MAXN || nd > ST_MAXD) return false;
  *nfull = nf;
  return true;
}

// A second stream per device, on which the strip kernel over the windows with NoData
// runs beside the one over the windows without (their items are disjoint): one after
// the other, two half-full waves of a small job would take two wave times.  Created
// once per device, outside any stream capture; each job forks and joins it with its
// own events.
static int side_stream(cudaStream_t* out) {
  static std::mutex mu;
  static cudaStream_t pool[64] = {};
  int dev = 0;
  FSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FSG_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(mu);
  if (!pool[dev]) FSG_CUDA(cudaStreamCreateWithFlags(&pool[dev], cudaStreamNonBlocking));
  *out = pool[dev];
  return FSG_OK;
}

// One topousm_fast strip-path job: host images of every device table (tile
// descriptors, strip items, Gaussian weight tables), the layout of its device
// buffer and the launch parameters.  The eager entry point uploads the images
// into stream-ordered scratch; a plan uploads them once into memory it owns.
// enqueue() issues only launches, memsets and event fork/join of the
// per-window decimation pipelines on the auxiliary streams (capturable).
struct TopoJob {
  TopoJob() = default;
  TopoJob(const TopoJob&) = delete;
  TopoJob& operator=(const TopoJob&) = delete;
  ~TopoJob() {
    if (TA) tc_release(TA);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
  }
  bool empty = true, fixed = false;
  // tensor-core path (fsg_topousm_tc.cu): its CTA tiles, the device-built list of
  // tiles with NoData that the exact kernel (kern) then computes, and its count
  bool tc = false;
  TcArgs* TA = nullptr;
  size_t tc_smem = 0, tci_off = 0, fix_off = 0, fixc_off = 0;
  std::vector<int4> tc_it;
  int ntiles = 0, nfull = 0, maxh = 1, maxw = 1, grid = 0;
  std::vector<TopoTileK> tk;
  std::vector<StripItem> items;
  // batched decimation: one DecItem per (window, decimated radius); consecutive
  // items with the same (f, rs, R) form launch chunks of at most nslots items,
  // item k of a chunk using scratch slot k
  struct DecRef {
    int t, slot;
    size_t gv, ms;  // floats into the weight table / bytes from the dec area
    bool zmax;      // this item's downsample also takes the window's max |z|
  };
  struct DecChunk {
    int first, count, maxhs, maxws, rs, R;
  };
  std::vector<DecItem> ditems;
  std::vector<DecRef> dref;
  std::vector<DecChunk> dchunks;
  bool absmax_fused = false;  // every window's max |z| comes from its downsample
  size_t slot_bytes = 0, slot_plane = 0;
  int nslots = 0;
  std::vector<float> gv, g1;
  std::vector<size_t> dec_ms;  // per (tile, dec), tile-major: byte offset of its coarse mean in the dec area
  size_t topo_bytes = 0, dec_bytes = 0, g1_off = 0, gv_off = 0, tiles_off = 0, items_off = 0, ditems_off = 0,
         dflags_off = 0, flags_off = 0, total = 0;
  StripArgs A;
  void (*kern)(StripArgs) = nullptr;
  // hybrid kernel split by the windows' NoData flags (split): kern = the items of windows
  // without NoData, kern2 = the others (and every item of the tensor path's fix-up list);
  // partition_items builds the two lists (A: clean, A2: the rest) on the device
  bool split = false;
  void (*kern2)(StripArgs) = nullptr;
  StripArgs A2;
  size_t part_off = 0;
  cudaStream_t side = nullptr;  // kern2 runs here, beside kern
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  size_t smem = 0;
  int threads = 0;  // block size (0: FX_NT for the fixed kernels, ST_NT otherwise)
  // bound device state
  char* base = nullptr;

  void bind(void* dev) {
    base = static_cast<char*>(dev);
    int* flags = reinterpret_cast<int*>(base + flags_off);
    for (int t = 0; t < ntiles; ++t) {
      tk[t].nan_flag = flags + t;
      for (int d = 0; d < tk[t].ndec; ++d) tk[t].dec[d].ms = nullptr;
    }
    // coarse means: per (tile, dec) in tile-major order
    size_t k = 0;
    for (int t = 0; t < ntiles; ++t)
      for (int d = 0; d < tk[t].ndec; ++d) tk[t].dec[d].ms = reinterpret_cast<float*>(base + topo_bytes + dec_ms[k++]);
    const float* g1d = reinterpret_cast<const float*>(base + g1_off);
    const float* gvd = reinterpret_cast<const float*>(base + gv_off);
    int* dflags = reinterpret_cast<int*>(base + dflags_off);
    for (size_t i = 0; i < ditems.size(); ++i) {
      DecItem& D = ditems[i];
      const DecRef& r = dref[i];
      char* sl = base + (size_t)r.slot * slot_bytes;
      D.z = tk[r.t].z;
      D.small = reinterpret_cast<float*>(sl);
      D.vm = reinterpret_cast<float*>(sl + slot_plane);
      D.wm = reinterpret_cast<float*>(sl + 2 * slot_plane);
      D.sw = reinterpret_cast<float*>(sl + 3 * slot_plane);
      D.ms = reinterpret_cast<float*>(base + topo_bytes + r.ms);
      D.gv = gvd + r.gv;
      D.g1 = g1d;
      D.flag = dflags + i;
      D.zmax = r.zmax ? reinterpret_cast<unsigned*>(flags + ntiles) : nullptr;
      D.tnan = r.zmax ? flags + r.t : nullptr;
    }
    A.tiles = reinterpret_cast<const TopoTileK*>(base + tiles_off);
    A.items = reinterpret_cast<const StripItem*>(base + items_off);
    A.zmax = reinterpret_cast<const unsigned*>(flags + ntiles);
    if (split && !tc) {  // the device-built lists of partition_items
      int* counts = reinterpret_cast<int*>(base + part_off);
      StripItem* lists = reinterpret_cast<StripItem*>(base + part_off + 256);
      const size_t stride = ((sizeof(StripItem) * items.size() + 255) & ~(size_t)255) / sizeof(StripItem);
      A2 = A;
      A.items = lists;
      A.nitems_dev = counts;
      A2.items = lists + stride;
      A2.nitems_dev = counts + 1;
    }
    if (tc) {
      StripItem* fix = reinterpret_cast<StripItem*>(base + fix_off);
      int* fixc = reinterpret_cast<int*>(base + fixc_off);
      A.items = fix;
      A.nitems_dev = fixc;
      tc_bind(TA, A.tiles, reinterpret_cast<const int4*>(base + tci_off), (int)tc_it.size(), fix, fixc,
              reinterpret_cast<unsigned*>(flags + ntiles));
    }
  }
  int upload(cudaStream_t s) const {
    if (!g1.empty()) FSG_UPLOAD(base + g1_off, g1.data(), g1.size() * sizeof(float), s);
    if (!gv.empty()) FSG_UPLOAD(base + gv_off, gv.data(), gv.size() * sizeof(float), s);
    FSG_UPLOAD(base + tiles_off, tk.data(), sizeof(TopoTileK) * ntiles, s);
    FSG_UPLOAD(base + items_off, items.data(), sizeof(StripItem) * items.size(), s);
    if (!ditems.empty())
      FSG_UPLOAD(base + ditems_off, ditems.data(), sizeof(DecItem) * ditems.size(), s);
    if (tc) FSG_UPLOAD(base + tci_off, tc_it.data(), sizeof(int4) * tc_it.size(), s);
    return FSG_OK;
  }

  // the decimated radii of every window: per chunk one launch per stage
  int enqueue_decimation(cudaStream_t s) const {
    const DecItem* dev = reinterpret_cast<const DecItem*>(base + ditems_off);
    for (const DecChunk& c : dchunks) {
      const DecItem* it = dev + c.first;
      const dim3 b2(32, 8);
      const dim3 g2((c.maxws + 31) / 32, (c.maxhs + 7) / 8, c.count);
      dec_downsample<<<g2, b2, 0, s>>>(it);
      // void fill (skipped on the device for grids without NaN cells; the grids of its
      // column and combine passes stride over rows, so a skipped pass is a few blocks)
      constexpr int FILL_ROW_BLOCKS = 64;
      dec_fill_cols<<<dim3((c.maxws + NT - 1) / NT, std::min(c.maxhs, FILL_ROW_BLOCKS), c.count), NT, 0, s>>>(it);
      int th, tw;
      size_t smem;
      row_geometry(c.R, 1, c.maxws, &th, &tw, &smem);
      if (smem > 48 * 1024) FSG_CUDA(cudaFuncSetAttribute(dec_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      dec_rows<<<dim3((c.maxws + tw - 1) / tw, (c.maxhs + th - 1) / th, c.count), NT, smem, s>>>(it, 0, th, tw);
      dec_fill<<<dim3(g2.x, std::min<unsigned>(g2.y, FILL_ROW_BLOCKS / 8), c.count), b2, 0, s>>>(it);
      // the radius's mean
      const int chunk = 128;  // rows per block of the box column pass (as launch_box)
      if (c.rs <= 1)
        dec_mean_cols<<<dim3((c.maxws + NT - 1) / NT, std::min(c.maxhs, 65535), c.count), NT, 0, s>>>(it, chunk);
      else
        dec_mean_cols<<<dim3((c.maxws + NT - 1) / NT, (c.maxhs + chunk - 1) / chunk, c.count), NT, 0, s>>>(it, chunk);
      row_geometry(c.rs <= 1 ? 4 : c.rs, 1, c.maxws, &th, &tw, &smem);
      if (smem > 48 * 1024) FSG_CUDA(cudaFuncSetAttribute(dec_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      dec_rows<<<dim3((c.maxws + tw - 1) / tw, (c.maxhs + th - 1) / th, c.count), NT, smem, s>>>(it, 1, th, tw);
      FSG_LAUNCHED(6);
    }
    return FSG_OK;
  }

  int enqueue(cudaStream_t s) const {
    if (empty) return FSG_OK;
    int* flags = reinterpret_cast<int*>(base + flags_off);
    const TopoTileK* tiles_dev = reinterpret_cast<const TopoTileK*>(base + tiles_off);
    FSG_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * (ntiles + 1), s));
    if (!ditems.empty()) {
      FSG_CUDA(cudaMemsetAsync(base + dflags_off, 0, sizeof(int) * ditems.size(), s));
      int st = enqueue_decimation(s);
      if (st) return st;
    }
    if (tc) {
      FSG_CUDA(cudaMemsetAsync(base + fixc_off, 0, sizeof(int), s));
      // The tensor kernel records max |z| of every input region it stages; with a
      // largest radius of 32 those regions are exactly what the exact kernel's strips
      // of the listed tiles read, otherwise the strips reach further and the windows
      // are scanned first (by the decimation's downsample when every window has one).
      if (A.R != 32 && !absmax_fused) {
        window_absmax<<<dim3(128, ntiles), 256, 0, s>>>(tiles_dev, reinterpret_cast<unsigned*>(flags + ntiles), flags);
        FSG_LAUNCHED(1);
      }
      timing_mark(s, true);
      int st2 = tc_launch(TA, tc_smem, s);
      timing_mark(s, false);
      if (st2) return st2;
      (split ? kern2 : kern)<<<grid, threads ? threads : FX_NT, smem, s>>>(A);  // the listed tiles, exact NaN-aware means
      FSG_LAUNCHED(1);
      return FSG_OK;
    }
    if (fixed) {
      if (!absmax_fused) {
        window_absmax<<<dim3(128, ntiles), 256, 0, s>>>(tiles_dev, reinterpret_cast<unsigned*>(flags + ntiles), flags);
        FSG_LAUNCHED(1);
      }
    } else {
      window_nan_flags<<<dim3(256, ntiles), 256, 0, s>>>(tiles_dev, flags);
      FSG_LAUNCHED(1);
    }
    if (split) {
      int* counts = reinterpret_cast<int*>(base + part_off);
      FSG_CUDA(cudaMemsetAsync(counts, 0, 2 * sizeof(int), s));
      const int n = (int)items.size();
      partition_items<<<(n + 255) / 256, 256, 0, s>>>(reinterpret_cast<const StripItem*>(base + items_off), n,
                                                      tiles_dev, const_cast<StripItem*>(A.items), counts,
                                                      const_cast<StripItem*>(A2.items), counts + 1);
      FSG_LAUNCHED(1);
      timing_mark(s, true);
      FSG_CUDA(cudaEventRecord(fork_ev, s));
      FSG_CUDA(cudaStreamWaitEvent(side, fork_ev, 0));
      kern<<<grid, threads, smem, s>>>(A);
      FSG_LAUNCHED(1);
      kern2<<<grid, threads, smem, side>>>(A2);
      FSG_LAUNCHED(1);
      FSG_CUDA(cudaEventRecord(join_ev, side));
      FSG_CUDA(cudaStreamWaitEvent(s, join_ev, 0));
      timing_mark(s, false);
      return FSG_OK;
    }
    if (fixed) timing_mark(s, true);
    kern<<<grid, threads ? threads : (fixed ? FX_NT : ST_NT), smem, s>>>(A);
    if (fixed) timing_mark(s, false);
    FSG_LAUNCHED(1);
    return FSG_OK;
  }
};

static int topousm_strip_prepare_exact(const float* raster_dev, int64_t ld, const fsg_tile* tiles, int32_t ntiles,
                                       const fsg_topousm_params* p, const fsg_plane* out, int nfull, TopoJob& J) {
  const std::vector<int> radii(p->radii, p->radii + p->nradii);
  J.ntiles = ntiles;
  J.nfull = nfull;
  for (int t = 0; t < ntiles; ++t) {
    J.maxh = std::max(J.maxh, tiles[t].win_h);
    J.maxw = std::max(J.maxw, tiles[t].win_w);
  }
  std::vector<int> dec_idx;
  for (int i = nfull; i < p->nradii; ++i) dec_idx.push_back(i);
  int R = 0;
  for (int i = 0; i < nfull; ++i) R = std::max(R, radii[i]);
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  // exact fixed-point kernel when its ring fits in shared memory, else the compensated one
  const int fx_ring = 2 * R + 2 * FX_G + 1;
  J.fixed = nfull >= 1 && nfull <= FX_MAXNR && 2 * R < FX_NT - 32 && FxSmem::bytes(fx_ring) <= di.smem_optin;
  const int TW = J.fixed ? FX_NT - 2 * R : ((ST_NT - 2 * R) / ST_SEG) * ST_SEG;
  const int CHUNK = J.fixed ? 1024 : 512;
  for (int t = 0; t < ntiles; ++t) {
    const fsg_tile& T = tiles[t];
    if (T.core_h == 0 || T.core_w == 0) continue;
    const int cy0 = T.core_y0 - T.win_y0, cx0 = T.core_x0 - T.win_x0;
    for (int x = cx0; x < cx0 + T.core_w; x += TW)
      for (int y = cy0; y < cy0 + T.core_h; y += CHUNK) J.items.push_back({t, x, y, std::min(y + CHUNK, cy0 + T.core_h)});
  }
  J.empty = J.items.empty();
  if (J.empty) return FSG_OK;
  // per (tile, dec) coarse means, void-fill weight tables and batched decimation items
  const size_t esz = out->dtype == FSG_F32 ? 4 : (out->dtype == FSG_I16 ? 2 : 1);
  J.tk.assign(ntiles, TopoTileK{});
  for (int t = 0; t < ntiles; ++t) {
    const fsg_tile& T = tiles[t];
    TopoTileK& k = J.tk[t];
    std::memset(&k, 0, sizeof(k));
    k.z = ZView{raster_dev + (long long)T.win_y0 * ld + T.win_x0, ld, T.win_h, T.win_w, (float)p->nodata,
                p->has_nodata != 0};
    k.cy0 = T.core_y0 - T.win_y0;
    k.cx0 = T.core_x0 - T.win_x0;
    k.ch = T.core_h;
    k.cw = T.core_w;
    k.gy0 = T.win_y0;
    k.gx0 = T.win_x0;
    k.out = static_cast<char*>(out->ptr) + ((long long)T.out_y0 * out->ld + T.out_x0) * esz;
    k.ndec = (int)dec_idx.size();
    for (size_t d = 0; d < dec_idx.size(); ++d) {
      const int r = radii[dec_idx[d]];
      const int f = topousm_downsample_factor((double)r, p->pixel_size);
      const int hs = std::max(1, (T.win_h + f - 1) / f), ws = std::max(1, (T.win_w + f - 1) / f);
      J.dec_ms.push_back(J.dec_bytes);
      if (T.core_h > 0 && T.core_w > 0) {
        double sigma = std::max(1.0, (double)std::min(hs, ws) / 64.0);
        int Rg;
        std::vector<float> gw = gaussian_weights(sigma, &Rg);
        if (Rg + 1 > 4096) return fail(FSG_ERR_UNSUPPORTED, "void-fill Gaussian radius %d too large", Rg);
        const size_t go = J.gv.size();
        J.gv.insert(J.gv.end(), gw.begin(), gw.end());
        J.gv.resize((J.gv.size() + 63) & ~(size_t)63);  // 256-byte aligned tables
        DecItem D;
        std::memset(&D, 0, sizeof(D));
        D.f = f;
        D.hs = hs;
        D.ws = ws;
        D.rs = std::max(1, (int)std::nearbyint((double)r / f));
        D.R = Rg;
        J.ditems.push_back(D);
        J.dref.push_back({t, 0, go, J.dec_bytes, d == 0});
      }
      J.dec_bytes += ((size_t)hs * ws * sizeof(float) + 255) & ~(size_t)255;
      k.dec[d].h = hs;
      k.dec[d].w = ws;
      k.dec[d].zy = T.win_h > 1 ? (double)(hs - 1) / (double)(T.win_h - 1) : 1.0;
      k.dec[d].zx = T.win_w > 1 ? (double)(ws - 1) / (double)(T.win_w - 1) : 1.0;
      k.dec[d].weight = (float)p->weights[dec_idx[d]];
    }
  }
  auto al = [](size_t n) { return (n + 255) & ~(size_t)255; };
  if (!J.ditems.empty()) {
    int Rg;
    J.g1 = gaussian_weights(1.0, &Rg);
    // launch chunks: runs of items with the same (f, rs, R) (the row passes' shared-memory
    // geometry follows the radius), at most nslots items each; scratch slots of four
    // hs x ws planes (small, vm, wm, sw), up to ~1 GiB in all
    int mh = 1, mw = 1;
    for (const DecItem& D : J.ditems) {
      mh = std::max(mh, D.hs);
      mw = std::max(mw, D.ws);
    }
    J.slot_plane = al((size_t)mh * mw * sizeof(float));
    J.slot_bytes = 4 * J.slot_plane;
    const int n = (int)J.ditems.size();
    J.nslots = (int)std::max<size_t>(1, std::min<size_t>((size_t)n, ((size_t)1 << 30) / J.slot_bytes));
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      const DecItem &x = J.ditems[a], &y = J.ditems[b];
      return std::make_tuple(x.f, x.rs, x.R) < std::make_tuple(y.f, y.rs, y.R);
    });
    std::vector<DecItem> di;
    std::vector<TopoJob::DecRef> dr;
    for (int i : order) {
      di.push_back(J.ditems[i]);
      dr.push_back(J.dref[i]);
    }
    J.ditems.swap(di);
    J.dref.swap(dr);
    for (int i = 0; i < n;) {
      const DecItem& D0 = J.ditems[i];
      TopoJob::DecChunk c{i, 0, 1, 1, D0.rs, D0.R};
      while (i < n && c.count < J.nslots && J.ditems[i].f == D0.f && J.ditems[i].rs == D0.rs &&
             J.ditems[i].R == D0.R) {
        J.dref[i].slot = c.count++;
        c.maxhs = std::max(c.maxhs, J.ditems[i].hs);
        c.maxws = std::max(c.maxws, J.ditems[i].ws);
        ++i;
      }
      if (c.count > 65535) return fail(FSG_ERR_UNSUPPORTED, "too many decimation items in one launch");
      J.dchunks.push_back(c);
    }
    // the windows' max |z| from their downsample when every window with work has one
    // (the per-window grids cover the whole window)
    J.absmax_fused = true;
  }
  J.topo_bytes = (size_t)J.nslots * J.slot_bytes;
  J.g1_off = al(J.topo_bytes + J.dec_bytes);
  J.gv_off = J.g1_off + al(J.g1.size() * sizeof(float) + 1);
  J.tiles_off = J.gv_off + al(J.gv.size() * sizeof(float) + 1);
  J.items_off = J.tiles_off + al(sizeof(TopoTileK) * ntiles);
  J.ditems_off = J.items_off + al(sizeof(StripItem) * J.items.size());
  J.dflags_off = J.ditems_off + al(sizeof(DecItem) * J.ditems.size());
  J.flags_off = J.dflags_off + al(sizeof(int) * J.ditems.size() + 1);
  // the split of the items by NoData (hybrid kernel): two counts, then the two lists
  J.part_off = al(J.flags_off + sizeof(int) * (ntiles + 1));
  J.total = J.part_off + 256 + 2 * al(sizeof(StripItem) * J.items.size()) + 256;
  StripArgs& A = J.A;
  std::memset(&A, 0, sizeof(A));
  A.nitems = (int)J.items.size();
  A.nr = nfull;
  A.R = R;
  A.TW = TW;
  for (int i = 0; i < nfull; ++i) {
    A.radii[i] = radii[i];
    A.weights[i] = (float)p->weights[i];
    A.fn[i] = (float)(2 * radii[i] + 1);
    A.rn[i] = 1.0f / A.fn[i];
  }
  A.field = p->coarse_dev;
  A.fld = p->coarse_ld;
  A.fh = p->coarse_h;
  A.fw = p->coarse_w;
  A.sy = p->coarse_dev ? (float)((double)p->coarse_h / (double)p->full_h) : 0.f;
  A.sx = p->coarse_dev ? (float)((double)p->coarse_w / (double)p->full_w) : 0.f;
  A.w_large = (float)p->w_large;
  A.scale = (float)p->scale;
  A.rscale = A.scale > 0.f ? 1.0f / A.scale : 0.f;
  A.old = out->ld;
  A.dtype = out->dtype;
  A.qa = out->q_a;
  A.qb = out->q_b;
  A.qmin = out->q_min;
  A.qmax = out->q_max;
  A.have_small = p->nradii > 0;
  A.ring = fx_ring;
  if (J.fixed && nfull >= 2) {
    // hybrid: the ring holds the smaller radii only, the largest takes per-group row buffers
    // 192 threads and 4-row groups (three CTAs per SM) when the strip has at most 192 output
    // columns, else 256 threads and 8-row groups (two CTAs per SM)
    const int Rs = radii[nfull - 2];
    const bool narrow = TW <= 192;
    const int HG = narrow ? 4 : 8;
    const int hy_ring = 2 * Rs + HG + 1;
    const size_t hsmem = HySmem::bytes(hy_ring, HG);
    if ((narrow ? 3 : 2) * (hsmem + 1024) <= (size_t)di.smem_per_sm && nfull <= HY_MAXNR) {
      // two launches over device-built item lists: the items of windows without NoData
      // (CLEAN arithmetic), then the rest; the tensor path's fix-up takes the general kernel
      if (narrow) {
        switch (nfull) {
          case 2: J.kern = topousm_hybrid<2, 192, 4, 3, true>; J.kern2 = topousm_hybrid<2, 192, 4, 3, false>;
                  J.split = true; break;
          case 3: J.kern = topousm_hybrid<3, 192, 4, 3, true>; J.kern2 = topousm_hybrid<3, 192, 4, 3, false>;
                  J.split = true; break;
          default: J.kern = topousm_hybrid<4, 192, 4, 3, true>; J.kern2 = topousm_hybrid<4, 192, 4, 3, false>;
                   J.split = true; break;
        }
      } else {
        switch (nfull) {
          case 2: J.kern = topousm_hybrid<2, 256, 8, 2, true>; J.kern2 = topousm_hybrid<2, 256, 8, 2, false>;
                  J.split = true; break;
          case 3: J.kern = topousm_hybrid<3, 256, 8, 2, true>; J.kern2 = topousm_hybrid<3, 256, 8, 2, false>;
                  J.split = true; break;
          default: J.kern = topousm_hybrid<4, 256, 8, 2, true>; J.kern2 = topousm_hybrid<4, 256, 8, 2, false>;
                   J.split = true; break;
        }
      }
      J.threads = narrow ? 192 : 256;
      A.ring = hy_ring;
      J.smem = hsmem;
      FSG_CUDA(cudaFuncSetAttribute(J.kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)J.smem));
      FSG_CUDA(cudaFuncSetAttribute(J.kern2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)J.smem));
      st = side_stream(&J.side);
      if (st) return st;
      FSG_CUDA(cudaEventCreateWithFlags(&J.fork_ev, cudaEventDisableTiming));
      FSG_CUDA(cudaEventCreateWithFlags(&J.join_ev, cudaEventDisableTiming));
      int per = 0;
      FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, J.kern, J.threads, J.smem));
      J.grid = std::min((int)J.items.size(), di.sms * std::max(1, per));
      return FSG_OK;
    }
  }
  if (J.fixed) {
    switch (nfull) {
      case 1: J.kern = topousm_fixed<1>; break;
      case 2: J.kern = topousm_fixed<2>; break;
      case 3: J.kern = topousm_fixed<3>; break;
      default: J.kern = topousm_fixed<4>; break;
    }
    J.smem = FxSmem::bytes(fx_ring);
    FSG_CUDA(cudaFuncSetAttribute(J.kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)J.smem));
    int per = 0;
    FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, J.kern, FX_NT, J.smem));
    J.grid = std::min((int)J.items.size(), di.sms * std::max(1, per));
    return FSG_OK;
  }
  J.smem = StripSmem::floats(std::max(1, nfull), TW) * sizeof(float);
  switch (nfull) {
    case 0: J.kern = topousm_strip<0>; break;
    case 1: J.kern = topousm_strip<1>; break;
    case 2: J.kern = topousm_strip<2>; break;
    case 3: J.kern = topousm_strip<3>; break;
    case 4: J.kern = topousm_strip<4>; break;
    case 5: J.kern = topousm_strip<5>; break;
    default: J.kern = topousm_strip<6>; break;
  }
  if (J.smem > 48 * 1024) FSG_CUDA(cudaFuncSetAttribute(J.kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)J.smem));
  int per_sm = 0;
  FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, J.kern, ST_NT, J.smem));
  J.grid = std::min((int)J.items.size(), di.sms * std::max(1, per_sm));
  return FSG_OK;
}

// The tensor-core path over the same job: its CTA tiles and the fix-up list
// after the exact job's device tables; the exact kernel (already chosen: the
// fixed-point hybrid or single-ring kernel) takes the listed tiles.
static int topousm_tc_setup(TopoJob& J, int nfull) {
  tc_items(J.tk.data(), J.ntiles, &J.tc_it);
  if (J.tc_it.empty()) return FSG_OK;
  const size_t n = J.tc_it.size();
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  J.tci_off = al(J.total);
  J.fix_off = J.tci_off + al(sizeof(int4) * n);
  J.fixc_off = J.fix_off + al(sizeof(StripItem) * n);
  J.total = J.fixc_off + 256;
  int st = tc_prepare(&J.TA, J.A, nfull, &J.tc_smem);
  if (st) return st;
  J.tc = true;
  return FSG_OK;
}

static int topousm_strip_prepare(const float* raster_dev, int64_t ld, const fsg_tile* tiles, int32_t ntiles,
                                 const fsg_topousm_params* p, const fsg_plane* out, int nfull, TopoJob& J) {
  int st = topousm_strip_prepare_exact(raster_dev, ld, tiles, ntiles, p, out, nfull, J);
  if (st || J.empty) return st;
  if (p->path == FSG_TOPOUSM_TENSOR && J.fixed && tc_supported(J.A.radii, nfull)) return topousm_tc_setup(J, nfull);
  return FSG_OK;
}

static int topousm_strip_path(const float* raster_dev, int64_t ld, const fsg_tile* tiles, int32_t ntiles,
                              const fsg_topousm_params* p, const fsg_plane* out, int nfull, cudaStream_t s) {
  TopoJob J;
  int st = topousm_strip_prepare(raster_dev, ld, tiles, ntiles, p, out, nfull, J);
  if (st || J.empty) return st;
  StreamScratch scratch;
  st = scratch.alloc(J.total, s);
  if (st) return st;
  J.bind(scratch.ptr);
  st = J.upload(s);
  if (st) return st;
  return J.enqueue(s);
}

struct TopoPlan final : fsg_plan {
  TopoJob J;
  void* dev = nullptr;
  ~TopoPlan() override {
    if (dev) cudaFree(dev);
  }
  int launch(cudaStream_t s) override { return J.enqueue(s); }
};



}  // namespace fsg

using namespace fsg;

static int topousm_validate(int64_t ld, int32_t raster_h, int32_t raster_w, const fsg_tile* tiles, int32_t ntiles,
                            const fsg_topousm_params* p, const fsg_plane* out) {
  if (!p || !out || (ntiles > 0 && !tiles)) return fail(FSG_ERR_INVALID, "null argument");
  if (ntiles < 0 || raster_h < 0 || raster_w < 0 || ld < raster_w) return fail(FSG_ERR_INVALID, "bad raster shape");
  if (!out->ptr) return fail(FSG_ERR_INVALID, "output plane is NULL");
  if (out->dtype < FSG_F32 || out->dtype > FSG_I16) return fail(FSG_ERR_DTYPE, "dtype %d", out->dtype);
  if (p->nradii < 0 || (p->nradii > 0 && (!p->radii || !p->weights)))
    return fail(FSG_ERR_INVALID, "radii/weights");
  if (p->nradii == 0 && !p->coarse_dev) return fail(FSG_ERR_INVALID, "no radius and no coarse field");
  for (int i = 0; i < p->nradii; ++i)
    if (p->radii[i] < 1) return fail(FSG_ERR_INVALID, "radius %d < 1", p->radii[i]);
  if (p->coarse_dev && (p->coarse_h < 1 || p->coarse_w < 1 || p->coarse_ld < p->coarse_w || p->full_h < 1 ||
                        p->full_w < 1))
    return fail(FSG_ERR_INVALID, "coarse field shape");
  return validate_tiles(raster_h, raster_w, tiles, ntiles, 1);
}

extern "C" int fsg_topousm_plan(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                                const fsg_tile* tiles, int32_t ntiles, const fsg_topousm_params* p,
                                const fsg_plane* out, fsg_plan** plan) {
  if (!plan) return fail(FSG_ERR_INVALID, "null plan pointer");
  *plan = nullptr;
  int st = topousm_validate(ld, raster_h, raster_w, tiles, ntiles, p, out);
  if (st) return st;
  const std::vector<int> rv(p->radii, p->radii + p->nradii);
  int nfull = 0;
  if (!strip_path_ok(rv, p->pixel_size, &nfull))
    return fail(FSG_ERR_UNSUPPORTED, "topousm plan: the radii must ascend with the full-resolution radii first");
  TopoPlan* P = new TopoPlan();
  st = topousm_strip_prepare(raster_dev, ld, tiles, ntiles, p, out, nfull, P->J);
  if (!st && !P->J.empty) {
    cudaError_t e = cudaMalloc(&P->dev, P->J.total);
    if (e != cudaSuccess) {
      P->dev = nullptr;
      st = cuda_fail(e, "cudaMalloc(plan)");
    } else {
      P->J.bind(P->dev);
      st = P->J.upload(nullptr);
      if (!st) {
        e = cudaStreamSynchronize(nullptr);
        if (e != cudaSuccess) st = cuda_fail(e, "plan upload");
      }
    }
  }
  if (st) {
    delete P;
    return st;
  }
  *plan = P;
  return FSG_OK;
}

extern "C" int fsg_topousm(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                           const fsg_tile* tiles, int32_t ntiles, const fsg_topousm_params* p,
                           const fsg_plane* out, void* stream) {
  int st = topousm_validate(ld, raster_h, raster_w, tiles, ntiles, p, out);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  {
    const std::vector<int> rv(p->radii, p->radii + p->nradii);
    int nfull = 0;
    if (strip_path_ok(rv, p->pixel_size, &nfull)) return topousm_strip_path(raster_dev, ld, tiles, ntiles, p, out, nfull, s);
  }
  int maxh = 1, maxw = 1;
  for (int t = 0; t < ntiles; ++t) {
    maxh = std::max(maxh, tiles[t].win_h);
    maxw = std::max(maxw, tiles[t].win_w);
  }
  StreamScratch scratch;
  st = scratch.alloc(TopoScratch::bytes(maxh, maxw), s);
  if (st) return st;
  TopoScratch S;
  S.carve(scratch.ptr, maxh, maxw);
  st = prepare_g1(S, s);
  if (st) return st;
  std::vector<int> radii(p->radii, p->radii + p->nradii);
  std::vector<float> weights(p->nradii);
  for (int i = 0; i < p->nradii; ++i) weights[i] = (float)p->weights[i];
  for (int t = 0; t < ntiles; ++t) {
    const fsg_tile& T = tiles[t];
    if (T.core_h == 0 || T.core_w == 0) continue;
    ZView z{raster_dev + (long long)T.win_y0 * ld + T.win_x0, ld, T.win_h, T.win_w, (float)p->nodata,
            p->has_nodata != 0};
    TopoScratch W = S;
    W.acc = resize(S.acc, T.win_h, T.win_w);
    W.vm = resize(S.vm, T.win_h, T.win_w);
    W.wm = resize(S.wm, T.win_h, T.win_w);
    if (p->nradii > 0) {
      st = topousm_window(z, radii, weights, p->pixel_size, W, s);
      if (st) return st;
    }
    FinalArgs A;
    std::memset(&A, 0, sizeof(A));
    A.z = z;
    A.acc = W.acc;
    A.have_small = p->nradii > 0;
    A.field = p->coarse_dev;
    A.fld = p->coarse_ld;
    A.fh = p->coarse_h;
    A.fw = p->coarse_w;
    A.sy = (float)((double)p->coarse_h / (double)p->full_h);
    A.sx = (float)((double)p->coarse_w / (double)p->full_w);
    A.w_large = (float)p->w_large;
    A.gy0 = T.win_y0;
    A.gx0 = T.win_x0;
    A.cy0 = T.core_y0 - T.win_y0;
    A.cx0 = T.core_x0 - T.win_x0;
    A.ch = T.core_h;
    A.cw = T.core_w;
    A.scale = (float)p->scale;
    size_t esz = out->dtype == FSG_F32 ? 4 : (out->dtype == FSG_I16 ? 2 : 1);
    A.out = static_cast<char*>(out->ptr) + ((long long)T.out_y0 * out->ld + T.out_x0) * esz;
    A.old = out->ld;
    A.dtype = out->dtype;
    A.qa = out->q_a;
    A.qb = out->q_b;
    A.qmin = out->q_min;
    A.qmax = out->q_max;
    Grid2 gd = grid2d(T.core_h, T.core_w);
    final_kernel<<<gd.g, gd.b, 0, s>>>(A);
    FSG_LAUNCHED(1);
  }
  return FSG_OK;
}

extern "C" int fsg_topousm_coarse_field(const float* coarse_dev, int64_t ld, int32_t h, int32_t w,
                                        const int32_t* radii, const double* weights, int32_t n,
                                        double decimation, float* field_dev, int64_t field_ld, void* stream) {
  if (!coarse_dev || !field_dev || n < 1 || !radii || !weights) return fail(FSG_ERR_INVALID, "null argument");
  if (h < 1 || w < 1 || ld < w || field_ld < w) return fail(FSG_ERR_INVALID, "bad shape");
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch scratch;
  int st = scratch.alloc(TopoScratch::bytes(2 * h, 2 * w), s);
  if (st) return st;
  TopoScratch S;
  S.carve(scratch.ptr, 2 * h, 2 * w);
  st = prepare_g1(S, s);
  if (st) return st;
  ZView z{coarse_dev, ld, h, w, 0.f, 0};
  AView field{field_dev, field_ld, h, w};
  AView mean = resize(S.acc, h, w);
  for (int i = 0; i < n; ++i) {
    // _impl_topousm_fast.py:147-154
    int rc = std::max(1, (int)std::nearbyint((double)radii[i] / std::max(decimation, 1.0)));
    st = mean_for_radius(z, rc, S, mean, s);
    if (st) return st;
    Grid2 gd = grid2d(h, w);
    field_accum<<<gd.g, gd.b, 0, s>>>(mean, (float)weights[i], i == 0, field);
    FSG_LAUNCHED(1);
  }
  return FSG_OK;
}

extern "C" int fsg_overview(const float* raster_dev, int64_t ld, int32_t h, int32_t w, double nodata,
                            int32_t has_nodata, float* out_dev, int32_t out_h, int32_t out_w, int64_t out_ld,
                            void* stream) {
  if (!raster_dev || !out_dev) return fail(FSG_ERR_INVALID, "null argument");
  if (h < 1 || w < 1 || out_h < 1 || out_w < 1 || out_h > h || out_w > w || ld < w || out_ld < out_w)
    return fail(FSG_ERR_INVALID, "bad shape");
  ZView z{raster_dev, ld, h, w, (float)nodata, has_nodata != 0};
  AView o{out_dev, out_ld, out_h, out_w};
  Grid2 gd = grid2d(out_h, out_w);
  overview_kernel<<<gd.g, gd.b, 0, (cudaStream_t)stream>>>(z, o);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_topousm_downsample_factor(double radius, double pixel_size) {
  return topousm_downsample_factor(radius, pixel_size);
}
