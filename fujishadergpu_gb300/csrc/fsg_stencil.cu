// Fused 3x3-class stencils: hillshade, slope and the four curvature products
// from one read of each halo window.
//
// Reference semantics, per tile window (algorithms/tile/dask_bridge.py:72-151):
//   handle_nan_for_gradient (_nan_utils.py:50-74): NaN cells are replaced by a
//     NaN-aware Gaussian(sigma=1, truncate 4, mode 'nearest') mean, computed
//     as two separable passes (axis 0 then axis 1) in float64 with a float32
//     intermediate, as scipy.ndimage.gaussian_filter does;
//   np.gradient(filled, |sy|, |sx|, edge_order=2): central differences inside
//     the window, second-order one-sided formulas on its first/last row/col;
//   hillshade (_impl_hillshade.py:20-54), slope (_impl_slope.py:19-35),
//   curvature with a second np.gradient on the SIGNED steps
//   (_impl_curvature.py:19-57); NaN restored at NoData cells.
//
// Work decomposition: every tile core is cut into TY x TX pixel blocks; a
// persistent grid walks the flattened (tile, block) list.  Each block stages
// its (TY+6) x (TX+8) halo region in shared memory (float4 loads when the
// rows are 16-byte aligned), takes the NaN-fill slow path only when a NaN
// lies in that region, computes dx/dy once into shared memory and emits all
// requested planes with 4-pixel vector stores.
#include <algorithm>
#include <array>
#include <mutex>
#include <cstring>
#include <vector>

#include <cuda.h>
#include <cstdlib>

#include "fsg_common.cuh"

namespace fsg {
namespace {

#ifndef FSG_STENCIL_MINB
#define FSG_STENCIL_MINB 1  // minimum resident blocks per SM requested from ptxas
#endif

constexpr int TX = 64, TY = 32, NT = 256;
constexpr int FHY = 3, FHX = 4;           // halo of the staged DEM region
constexpr int FR = TY + 2 * FHY;          // 38 rows
constexpr int FC = TX + 2 * FHX;          // 72 cols
constexpr int DHY = 2, DHX = 2;           // halo of the dx/dy region
constexpr int DR = TY + 2 * DHY;          // 36
constexpr int DC = TX + 2 * DHX;          // 68
constexpr int WHY = FHY + 4, WHX = FHX + 4;  // +4: reach of the 9-tap Gaussian fill
constexpr int WR = TY + 2 * WHY;          // 46
constexpr int WC = TX + 2 * WHX;          // 80
constexpr int INLINE_TILES = 8;

constexpr size_t SMEM_F = sizeof(float) * FR * FC;
constexpr size_t SMEM_D = sizeof(float) * 2 * DR * DC;
constexpr size_t SMEM_FILL = sizeof(float) * (WR * WC + 2 * FR * WC) + 4 * sizeof(unsigned) * FR * 3;
constexpr size_t SMEM_BYTES = SMEM_F + (SMEM_D > SMEM_FILL ? SMEM_D : SMEM_FILL);

// np.gradient constants along one axis for one step size (float32, as NumPy
// applies the Python-float coefficients to float32 arrays).
struct Axis {
  float d2, rcp;      // central: (f[+1] - f[-1]) / d2, d2 = f32(2*step), rcp = RN(1/d2)
  float fa, fb, fc;   // first index:  fa*f0 + fb*f1 + fc*f2
  float ba, bb, bc;   // last index:   ba*f[-2] + bb*f[-1] + bc*f0
};

struct TileK {
  int wy0, wx0, wy1, wx1;   // window [y0, y1) x [x0, x1)
  int cy0, cx0, cy1, cx1;   // core
  int oy0, ox0;             // plane coords of (cy0, cx0)
  int nbx, block0;
  Axis g1x, g1y;            // first derivatives: |step| (handle_nan_for_gradient)
  Axis c2x, c2y;            // second derivatives: signed steps (compute_curvature_block)
  float sign_x, sign_y;     // hillshade east/north orientation
};

struct PlaneK {
  void* ptr;
  long long ld;
  int dtype, qmin, qmax;
  float qa, qb;
};

struct StencilArgs {
  const float* raster;
  long long ld;
  int rh, rw;
  const TileK* tiles_dev;
  int ntiles, total_blocks;
  float lx, ly, lz, z;
  int z_is_one;
  float ndf;
  int has_nodata;
  int slope_unit;
  unsigned outmask;
  float gw_hi[5], gw_lo[5];  // scipy Gaussian(sigma=1, radius 4) weights as float-float, [0] = centre
  unsigned char* block_flags;  // per (tile, block): nonzero = process; NULL = every block
  PlaneK planes[FSG_STENCIL_NOUT];
  TileK inl[INLINE_TILES];
};

// Derivative of a line at index k of a window [lo, hi); f(o) = value at k+o.
template <class Fn>
__device__ __forceinline__ float deriv(const Axis& a, int k, int lo, int hi, Fn f) {
  if (k > lo && k < hi - 1) return div_by(fsub(f(1), f(-1)), a.d2, a.rcp);
  if (k == lo) return fadd(fadd(fmul(a.fa, f(0)), fmul(a.fb, f(1))), fmul(a.fc, f(2)));
  return fadd(fadd(fmul(a.ba, f(-2)), fmul(a.bb, f(-1))), fmul(a.bc, f(0)));
}

__device__ __forceinline__ float gamma_display(float k) {
  // ((tanh(100k) + 1) / 2) ** (1/2.2) == (1 + exp(-200k)) ** (-1/2.2): three
  // hardware approximations (absolute error ~1e-7 on [0, 1]).  Where tanh
  // rounds to within a few float32 ulps of -1 the reference's own value is
  // quantised by that rounding; this form gives the unquantised value.
  float e = ex2_approx(k * -288.53900817779268f);  // exp(-200k) = 2^(-200 k log2(e))
  return ex2_approx(-0.45454545454545453f * lg2_approx(1.0f + e));
}

__device__ __forceinline__ float slope_value(float p, float q, int unit) {
  float g = __fsqrt_rn(fadd(fmul(p, p), fmul(q, q)));
  float r = atanf(g);
  if (unit == FSG_SLOPE_DEGREE) return fmul(r, 57.295780181884765625f);  // f32(180/pi)
  if (unit == FSG_SLOPE_PERCENT) return fmul(tanf(r), 100.0f);
  return r;
}


// Loads rows [gy0, gy0+R) x cols [gx0, gx0+C) of the raster into S (row pitch
// C), NoData -> NaN, cells outside the raster -> 0.  Returns true if this
// thread saw a NaN inside the window.
// Stages rows [gy0, gy0+R) x cols [gx0, gx0+C) of the raster in shared memory
// (row pitch C).  issue() starts every global load of the calling thread
// (float4 when the rows are 16-byte aligned) into registers; commit() maps
// NoData to NaN, stores to shared memory and reports whether this thread saw
// a NaN inside the window.  Splitting the two lets a block prefetch the next
// block's halo while it computes the current one.  Cells outside the raster
// read as 0 (they lie outside every window and are never used).
template <int R, int C>
struct Region {
  static constexpr int C4 = C / 4, N = R * C4, ITER = (N + NT - 1) / NT;
  float4 v[ITER];
  int gy0, gx0;

  __device__ __forceinline__ void issue(const StencilArgs& A, int y0, int x0) {
    gy0 = y0;
    gx0 = x0;
    const bool vec = ((reinterpret_cast<uintptr_t>(A.raster) & 15) == 0) && ((A.ld & 3) == 0) && ((x0 & 3) == 0);
#pragma unroll
    for (int k = 0; k < ITER; ++k) {
      const int i = threadIdx.x + k * NT;
      float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
      if (i < N) {
        const int r = i / C4, c = (i - (i / C4) * C4) * 4;
        const int gy = y0 + r, gx = x0 + c;
        if (gy >= 0 && gy < A.rh) {
          const float* row = A.raster + (long long)gy * A.ld;
          if (vec && gx >= 0 && gx + 3 < A.rw) {
            t = __ldg(reinterpret_cast<const float4*>(row + gx));
          } else {
            if (gx >= 0 && gx < A.rw) t.x = __ldg(row + gx);
            if (gx + 1 >= 0 && gx + 1 < A.rw) t.y = __ldg(row + gx + 1);
            if (gx + 2 >= 0 && gx + 2 < A.rw) t.z = __ldg(row + gx + 2);
            if (gx + 3 >= 0 && gx + 3 < A.rw) t.w = __ldg(row + gx + 3);
          }
        }
      }
      v[k] = t;
    }
  }

  __device__ __forceinline__ bool commit(const StencilArgs& A, const TileK& T, float* S) const {
    bool saw_nan = false;
    const bool hn = A.has_nodata != 0;
#pragma unroll
    for (int k = 0; k < ITER; ++k) {
      const int i = threadIdx.x + k * NT;
      if (i >= N) break;
      const int r = i / C4, c = (i - (i / C4) * C4) * 4;
      float e[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
      bool any = false;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (is_nodata(e[q], A.ndf, hn)) {
          e[q] = __int_as_float(0x7fc00000);
          any = true;
        }
      }
      if (any) {
        const int gy = gy0 + r, gx = gx0 + c;
        if (gy >= T.wy0 && gy < T.wy1) {
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (e[q] != e[q] && gx + q >= T.wx0 && gx + q < T.wx1) saw_nan = true;
        }
      }
      *reinterpret_cast<float4*>(S + r * C + c) = make_float4(e[0], e[1], e[2], e[3]);
    }
    return saw_nan;
  }
};

// The 9-tap symmetric Gaussian sums of two tap sets at once (the values and the valid
// mask of one cell), in float-float on the paired FP32 instructions: per set
// x[4] w0, then the pairs (x[4-k] + x[4+k]) wk from k = 4 inwards (scipy's symmetric
// correlate1d order), rounded once to float32.
__device__ __forceinline__ float2 gsum_ff2(const FF* w, const float* a, const float* b) {
  FF2 acc = ff_mul2({make_float2(a[4], b[4]), make_float2(0.f, 0.f)}, make_float2(w[0].hi, w[0].hi),
                    make_float2(w[0].lo, w[0].lo));
#pragma unroll
  for (int k = 4; k >= 1; --k)
    acc = ff_add2(acc, ff_mul2(two_sum2(make_float2(a[4 - k], b[4 - k]), make_float2(a[4 + k], b[4 + k])),
                               make_float2(w[k].hi, w[k].hi), make_float2(w[k].lo, w[k].lo)));
  return p_add(acc.hi, acc.lo);
}


// Output products of one pixel from its derivatives.  Hillshade, slope and
// the curvature formulas use hardware approximations of sqrt/rcp (relative
// error ~1e-7, far inside the 1e-5 x range parity bound); tanh is CUDA's tanhf,
// the function the reference's cp.tanh evaluates.
struct Light {
  float lx, ly, lz;
  int slope_unit;
};

__device__ __forceinline__ void pixel_products(const Light& L, float sign_x, float sign_y, unsigned om, float p,
                                               float q, float pz, float qz, float dxx, float dxy, float dyy,
                                               float dyx, float* o) {
  if (om & (1u << FSG_OUT_HILLSHADE)) {
    float e = pz * sign_x, nn = qz * sign_y;
    float hs = fadd(fadd(-fmul(e, L.lx), -fmul(nn, L.ly)), L.lz) * rsqrtf(fadd(fadd(fmul(e, e), fmul(nn, nn)), 1.0f));
    o[FSG_OUT_HILLSHADE] = fminf(fmaxf(hs, 0.0f), 1.0f);
  }
  if (om & (1u << FSG_OUT_SLOPE)) {
    float g2 = fadd(fmul(p, p), fmul(q, q));
    if (L.slope_unit == FSG_SLOPE_DEGREE) o[FSG_OUT_SLOPE] = atan_poly(sqrt_approx(g2)) * 57.295780181884765625f;
    else o[FSG_OUT_SLOPE] = slope_value(p, q, L.slope_unit);
  }
  if (om & ((1u << FSG_OUT_CURV_MEAN) | (1u << FSG_OUT_CURV_GAUSSIAN) | (1u << FSG_OUT_CURV_PLANFORM) |
            (1u << FSG_OUT_CURV_PROFILE))) {
    float p2 = fmul(p, p), q2 = fmul(q, q), tpq = fmul(fmul(2.0f, p), q);
    float g2 = fadd(p2, q2), one_g2 = fadd(1.0f, g2);
    float s15 = one_g2 * sqrt_approx(one_g2);  // (1 + p^2 + q^2)^1.5
    // numerators in NumPy's float32 order, every operation rounded (their terms cancel)
    if (om & (1u << FSG_OUT_CURV_MEAN)) {
      float s = fmul(fadd(dxy, dyx), 0.5f);
      float num = fadd(fsub(fmul(fadd(1.0f, q2), dxx), fmul(tpq, s)), fmul(fadd(1.0f, p2), dyy));
      o[FSG_OUT_CURV_MEAN] = gamma_display(-num * rcp_approx(2.0f * s15 + 1e-10f));
    }
    if (om & (1u << FSG_OUT_CURV_GAUSSIAN))
      o[FSG_OUT_CURV_GAUSSIAN] = gamma_display(fsub(fmul(dxx, dyy), fmul(dxy, dxy)) * rcp_approx(one_g2 * one_g2));
    if (om & (1u << FSG_OUT_CURV_PLANFORM)) {
      float num = fadd(fsub(fmul(q2, dxx), fmul(tpq, dxy)), fmul(p2, dyy));
      o[FSG_OUT_CURV_PLANFORM] = gamma_display(-num * rcp_approx(g2 * sqrt_approx(g2) + 1e-10f));
    }
    if (om & (1u << FSG_OUT_CURV_PROFILE)) {
      float num = fadd(fadd(fmul(p2, dxx), fmul(tpq, dxy)), fmul(q2, dyy));
      o[FSG_OUT_CURV_PROFILE] = gamma_display(-num * rcp_approx(g2 * s15 + 1e-10f));
    }
  }
  o[FSG_OUT_DX] = p;
  o[FSG_OUT_DY] = q;
}

// dx/dy over the (TY+4) x (TX+4) region; INTERIOR: the whole staged region lies
// inside the window, so every derivative is a central difference.
template <bool INTERIOR>
__device__ __forceinline__ void stage_first_derivs(const TileK& T, const float* F, float* DX, float* DY, int y0,
                                                   int x0) {
  constexpr int SR = NT / DC, SC = NT % DC;
  int r = threadIdx.x / DC, c = threadIdx.x % DC;
  for (int i = threadIdx.x; i < DR * DC; i += NT, r += SR, c += SC) {
    if (c >= DC) {
      c -= DC;
      ++r;
    }
    const float* f = F + (r + FHY - DHY) * FC + (c + FHX - DHX);
    if (INTERIOR) {
      DX[i] = div_by(fsub(f[1], f[-1]), T.g1x.d2, T.g1x.rcp);
      DY[i] = div_by(fsub(f[FC], f[-FC]), T.g1y.d2, T.g1y.rcp);
    } else {
      int gy = y0 - DHY + r, gx = x0 - DHX + c;
      if (gy < T.wy0 || gy >= T.wy1 || gx < T.wx0 || gx >= T.wx1) continue;
      DX[i] = deriv(T.g1x, gx, T.wx0, T.wx1, [&](int o) { return f[o]; });
      DY[i] = deriv(T.g1y, gy, T.wy0, T.wy1, [&](int o) { return f[o * FC]; });
    }
  }
}

// Per-pixel stage: thread = one column of the block, 8 consecutive rows, so a
// warp touches 32 consecutive shared-memory words and stores 32 consecutive
// output pixels of a row.
template <bool CURV, bool INTERIOR>
__device__ __forceinline__ void stage_pixels(const StencilArgs& A, const TileK& T, unsigned om, const float* F,
                                             const float* DX, const float* DY, int y0, int x0, unsigned nanbits) {
  const int j = threadIdx.x & (TX - 1);
  const int i0 = (threadIdx.x / TX) * (TY * TX / NT);
  const int gx = x0 + j;
  if (gx >= T.cx1) return;
  const long long pcol = (long long)(T.ox0 + gx - T.cx0);
  const long long prow0 = (long long)(T.oy0 + y0 + i0 - T.cy0);
  char* optr[FSG_STENCIL_NOUT];
  long long ostep[FSG_STENCIL_NOUT];
#pragma unroll
  for (int k = 0; k < FSG_STENCIL_NOUT; ++k) {
    const PlaneK& P = A.planes[k];
    const int esz = P.dtype == FSG_F32 ? 4 : (P.dtype == FSG_I16 ? 2 : 1);
    optr[k] = static_cast<char*>(P.ptr) + (prow0 * P.ld + pcol) * esz;
    ostep[k] = P.ld * esz;
  }
#pragma unroll 1
  for (int ii = 0; ii < TY * TX / NT; ++ii) {
    const int i = i0 + ii;
    const int gy = y0 + i;
    if (gy >= T.cy1) break;
    float o[FSG_STENCIL_NOUT];
    if ((nanbits >> ii) & 1u) {
#pragma unroll
      for (int k = 0; k < FSG_STENCIL_NOUT; ++k) o[k] = __int_as_float(0x7fc00000);
    } else {
      const float* f = F + (i + FHY) * FC + (j + FHX);
      float p, q, dxx = 0.f, dxy = 0.f, dyy = 0.f, dyx = 0.f;
      const float* dxp = DX + (i + DHY) * DC + j + DHX;
      const float* dyp = DY + (i + DHY) * DC + j + DHX;
      if (CURV) {
        p = dxp[0];
        q = dyp[0];
        if (INTERIOR) {
          dxx = div_by(fsub(dxp[1], dxp[-1]), T.c2x.d2, T.c2x.rcp);
          dxy = div_by(fsub(dxp[DC], dxp[-DC]), T.c2y.d2, T.c2y.rcp);
          dyy = div_by(fsub(dyp[DC], dyp[-DC]), T.c2y.d2, T.c2y.rcp);
          if (om & (1u << FSG_OUT_CURV_MEAN)) dyx = div_by(fsub(dyp[1], dyp[-1]), T.c2x.d2, T.c2x.rcp);
        } else {
          dxx = deriv(T.c2x, gx, T.wx0, T.wx1, [&](int o2) { return dxp[o2]; });
          dxy = deriv(T.c2y, gy, T.wy0, T.wy1, [&](int o2) { return dxp[o2 * DC]; });
          dyy = deriv(T.c2y, gy, T.wy0, T.wy1, [&](int o2) { return dyp[o2 * DC]; });
          if (om & (1u << FSG_OUT_CURV_MEAN))
            dyx = deriv(T.c2x, gx, T.wx0, T.wx1, [&](int o2) { return dyp[o2]; });
        }
      } else if (INTERIOR) {
        p = div_by(fsub(f[1], f[-1]), T.g1x.d2, T.g1x.rcp);
        q = div_by(fsub(f[FC], f[-FC]), T.g1y.d2, T.g1y.rcp);
      } else {
        p = deriv(T.g1x, gx, T.wx0, T.wx1, [&](int o2) { return f[o2]; });
        q = deriv(T.g1y, gy, T.wy0, T.wy1, [&](int o2) { return f[o2 * FC]; });
      }
      float pz = p, qz = q;
      if ((om & (1u << FSG_OUT_HILLSHADE)) && !A.z_is_one) {
        const float z = A.z;
        if (INTERIOR) {
          pz = div_by(fsub(fmul(f[1], z), fmul(f[-1], z)), T.g1x.d2, T.g1x.rcp);
          qz = div_by(fsub(fmul(f[FC], z), fmul(f[-FC], z)), T.g1y.d2, T.g1y.rcp);
        } else {
          pz = deriv(T.g1x, gx, T.wx0, T.wx1, [&](int o2) { return fmul(f[o2], z); });
          qz = deriv(T.g1y, gy, T.wy0, T.wy1, [&](int o2) { return fmul(f[o2 * FC], z); });
        }
      }
      const Light L{A.lx, A.ly, A.lz, A.slope_unit};
      pixel_products(L, T.sign_x, T.sign_y, om, p, q, pz, qz, dxx, dxy, dyy, dyx, o);
    }
#pragma unroll
    for (int k = 0; k < FSG_STENCIL_NOUT; ++k) {
      if (!(om & (1u << k))) continue;
      const PlaneK& P = A.planes[k];
      char* dst = optr[k] + ii * ostep[k];
      if (P.dtype == FSG_F32) *reinterpret_cast<float*>(dst) = o[k];
      else if (P.dtype == FSG_U8) *reinterpret_cast<uint8_t*>(dst) = (uint8_t)(int)quantize(o[k], P.qa, P.qb, P.qmin, P.qmax);
      else *reinterpret_cast<int16_t*>(dst) = (int16_t)(int)quantize(o[k], P.qa, P.qb, P.qmin, P.qmax);
    }
  }
}

// FIXED != 0: the output mask is known at compile time (unrequested planes are
// compiled out); FIXED == 0 reads it from the arguments.
template <bool CURV, unsigned FIXED>
__global__ void __launch_bounds__(NT, FSG_STENCIL_MINB) stencil_kernel(const __grid_constant__ StencilArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* F = reinterpret_cast<float*>(smem);                       // [FR][FC]
  unsigned char* U = smem + SMEM_F;
  float* DX = reinterpret_cast<float*>(U);                         // [DR][DC]
  float* DY = DX + DR * DC;
  float* W = reinterpret_cast<float*>(U);                          // [WR][WC] (fill path)
  float* VV = W + WR * WC;                                         // [FR][WC]
  float* VW = VV + FR * WC;                                        // [FR][WC]
  unsigned* vmask = reinterpret_cast<unsigned*>(VW + FR * WC);    // [FR][3] valid cells (fill path)
  unsigned* nmask = vmask + FR * 3;                                // [FR][3] NaN cells
  unsigned* needm = nmask + FR * 3;                                // [FR][3] needed NaN cells
  unsigned* wantm = needm + FR * 3;                                // [FR][3] wanted axis-0 columns

  const TileK* tiles = A.ntiles <= INLINE_TILES ? A.inl : A.tiles_dev;
  const int tid = threadIdx.x;
  const unsigned om = FIXED ? FIXED : A.outmask;

  // Block geometry of a flat block index.
  auto locate = [&](int blk, int* t_out, int* y0_out, int* x0_out) {
    int lo = 0, hi = A.ntiles - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (tiles[mid].block0 <= blk) lo = mid; else hi = mid - 1;
    }
    const TileK& Tl = tiles[lo];
    const int lb = blk - Tl.block0;
    const int by = lb / Tl.nbx, bx = lb - (lb / Tl.nbx) * Tl.nbx;
    *t_out = lo;
    *y0_out = Tl.cy0 + by * TY;
    *x0_out = Tl.cx0 + bx * TX;
  };

  for (int blk = blockIdx.x; blk < A.total_blocks; blk += gridDim.x) {
    if (A.block_flags && !A.block_flags[blk]) continue;  // the fast pass produced this block exactly
    int t_cur, y0, x0;
    locate(blk, &t_cur, &y0, &x0);
    const TileK& T = tiles[t_cur];
    const int fy0 = y0 - FHY, fx0 = x0 - FHX;
    const bool interior = fy0 >= T.wy0 && fy0 + FR <= T.wy1 && fx0 >= T.wx0 && fx0 + FC <= T.wx1;

    __syncthreads();  // the previous block is done with shared memory
    Region<FR, FC> halo;
    halo.issue(A, fy0, fx0);
    bool saw = halo.commit(A, T, F);
    const int any_nan = __syncthreads_or(saw);

    // NoData flags of this thread's 8 core pixels, before the fill rewrites F.
    unsigned nanbits = 0;
    {
      const int j = tid & (TX - 1);
      const int i0 = (tid / TX) * (TY * TX / NT);
#pragma unroll
      for (int ii = 0; ii < TY * TX / NT; ++ii) {
        float v = F[(FHY + i0 + ii) * FC + FHX + j];
        if (v != v) nanbits |= 1u << ii;
      }
    }

    if (any_nan) {
      // (a) row bitmasks over the 72 staged columns: in-window valid cells and
      //     in-window NaN cells
      for (int i = tid; i < FR * 3; i += NT) {
        const int r = i / 3, k = i - (i / 3) * 3;
        const int gy = fy0 + r;
        unsigned vb = 0, nb = 0;
        if (gy >= T.wy0 && gy < T.wy1) {
          for (int b = 0; b < 32; ++b) {
            const int c = 32 * k + b, gx = fx0 + c;
            if (c >= FC || gx < T.wx0 || gx >= T.wx1) continue;
            const float v = F[r * FC + c];
            if (v == v) vb |= 1u << b; else nb |= 1u << b;
          }
        }
        vmask[i] = vb;
        nmask[i] = nb;
      }
      __syncthreads();
      // (b) needed NaN cells: a valid cell within Chebyshev distance 3 (whose
      //     stencil may read the fill value); wanted axis-0 columns: within 8
      //     columns to the right of a needed cell (in the wide region's columns)
      for (int r = tid; r < FR; r += NT) {
        unsigned long long dil_lo = 0, dil_hi = 0;  // 96-bit OR of valid rows r-3..r+3, dilated by 3 columns
        for (int dr = -3; dr <= 3; ++dr) {
          const int rr = r + dr;
          if (rr < 0 || rr >= FR) continue;
          dil_lo |= (unsigned long long)vmask[rr * 3] | ((unsigned long long)vmask[rr * 3 + 1] << 32);
          dil_hi |= vmask[rr * 3 + 2];
        }
        unsigned long long d_lo = dil_lo, d_hi = dil_hi;
        for (int s1 = 1; s1 <= 3; ++s1) {
          d_lo |= (dil_lo << s1) | (dil_lo >> s1) | (dil_hi << (64 - s1));
          d_hi |= (dil_hi << s1) | (dil_hi >> s1) | (dil_lo >> (64 - s1));
        }
        const unsigned long long n_lo = ((unsigned long long)nmask[r * 3] | ((unsigned long long)nmask[r * 3 + 1] << 32)) & d_lo;
        const unsigned long long n_hi = nmask[r * 3 + 2] & d_hi;
        needm[r * 3] = (unsigned)n_lo;
        needm[r * 3 + 1] = (unsigned)(n_lo >> 32);
        needm[r * 3 + 2] = (unsigned)n_hi;
        unsigned long long w_lo = 0, w_hi = 0;  // W column xc = F column c + d, d = 0..8
        for (int d = 0; d <= 8; ++d) {
          w_lo |= n_lo << d;
          w_hi |= (n_hi << d) | (d ? (n_lo >> (64 - d)) : 0ull);
        }
        wantm[r * 3] = (unsigned)w_lo;
        wantm[r * 3 + 1] = (unsigned)(w_lo >> 32);
        wantm[r * 3 + 2] = (unsigned)w_hi;
      }
      // (c) the wider region the 9x9 Gaussian reaches
      {
        Region<WR, WC> wide;
        wide.issue(A, y0 - WHY, x0 - WHX);
        wide.commit(A, T, W);
      }
      __syncthreads();
      FF gw[5];
#pragma unroll
      for (int j = 0; j < 5; ++j) gw[j] = {A.gw_hi[j], A.gw_lo[j]};
      // (d) axis-0 pass (values and valid weights) at the wanted columns,
      //     'nearest' clamping at the window rows
      for (int i = tid; i < FR * WC; i += NT) {
        const int r = i / WC, xc = i - (i / WC) * WC;
        if (!((wantm[r * 3 + (xc >> 5)] >> (xc & 31)) & 1u)) continue;
        const int gy = fy0 + r, gx = x0 - WHX + xc;
        if (gy < T.wy0 || gy >= T.wy1 || gx < T.wx0 || gx >= T.wx1) continue;
        float xv[9], xw[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int yy = min(max(gy + j - 4, T.wy0), T.wy1 - 1);
          const float v = W[(yy - (y0 - WHY)) * WC + xc];
          const bool ok = v == v;
          xv[j] = ok ? v : 0.f;
          xw[j] = ok ? 1.f : 0.f;
        }
        const float2 sw2 = gsum_ff2(gw, xv, xw);
        VV[r * WC + xc] = sw2.x;
        VW[r * WC + xc] = sw2.y;
      }
      __syncthreads();
      // (e) axis-1 pass and the normalised fill value of each needed cell
      for (int i = tid; i < FR * FC; i += NT) {
        const int r = i / FC, c = i - (i / FC) * FC;
        if (!((needm[r * 3 + (c >> 5)] >> (c & 31)) & 1u)) continue;
        const int gx = fx0 + c;
        float xv[9], xw[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int xx = min(max(gx + j - 4, T.wx0), T.wx1 - 1);
          const int xc = xx - (x0 - WHX);
          xv[j] = VV[r * WC + xc];
          xw[j] = VW[r * WC + xc];
        }
        const float2 s2 = gsum_ff2(gw, xv, xw);
        const float sv = s2.x, sw = s2.y;
        F[i] = sw > 0.0f ? __fdiv_rn(sv, sw) : 0.0f;
      }
      __syncthreads();
    }

    if (CURV) {
      if (interior) stage_first_derivs<true>(T, F, DX, DY, y0, x0);
      else stage_first_derivs<false>(T, F, DX, DY, y0, x0);
      __syncthreads();
    }
    if (interior) stage_pixels<CURV, true>(A, T, om, F, DX, DY, y0, x0, nanbits);
    else stage_pixels<CURV, false>(A, T, om, F, DX, DY, y0, x0, nanbits);
  }
}


// ------------------------------------------------------------ fast pass
// Streaming kernel for the common case: a warp owns a strip of SW = 60 output
// columns and SH rows; lane l holds the column pair (x0 - 2 + 2l, x0 - 1 + 2l)
// as a float2, walks down the rows keeping f, dx, dy of the neighbouring rows
// in registers, and takes the horizontal neighbours from one warp shuffle each
// way per pair (lanes 1..30 emit outputs).  The arithmetic runs on both
// columns at once with the paired FP32 instructions of sm_100+ (FADD2, FMUL2,
// FFMA2: per component the same correctly rounded operation as the scalar
// form).  No shared memory, no barriers.  A unit that touches a window edge,
// or holds a valid pixel whose stencil reaches NoData (NaN propagates into its
// derivatives), is appended to a list; the fix-up kernel recomputes every
// listed unit exactly (NaN fill, one-sided edge formulas), as two halves of
// FW = 30 columns.
constexpr int SW = 128, SH = 64, FW = 32, NQ = SW / FW;  // unit 128 x 64; fix-up in quarters of 32 columns
// ring row: columns x0-4 .. x0+131 (the unit's 128 columns at offset 4, its halo x0-2, x0-1 at 2, 3
// and x0+128, x0+129 at 132, 133), one tensor-copy box; rows 640 bytes apart (128-byte aligned)
constexpr int RBOX = SW + 8, RW = 160;

struct FastTile {
  int wy0, wx0, wy1, wx1, cy0, cx0, cy1, cx1, oy0, ox0;
  int nstrip, unit0;   // strips across the core, first flat unit index
  Axis g1x, g1y, c2x, c2y;
  float sx, sy;
};

struct FastArgs {
  const float* raster;
  long long ld;
  float lx, ly, lz, z;
  int z_is_one;
  float ndf;
  int has_nodata;
  int slope_unit;
  const FastTile* tiles;
  int ntiles, total_units;
  unsigned* fix_list;   // unit quarters for the fix-up pass: unit | quarter << 28 | FIX_BAND
  unsigned* fix_count;  // number of entries in fix_list
  unsigned* queue;      // work queue: next unit of the flattened tile list (zeroed per launch)
  unsigned* fix_queue;  // work queue of the fix-up pass: next entry of fix_list (zeroed per launch)
  FF gw[5];                   // Gaussian fill weights (float-float)
  PlaneK planes[FSG_STENCIL_NOUT];
  int use_tma;                // tmap describes the raster (16-byte aligned base and row pitch)
  CUtensorMap tmap;           // 2-D float32 raster, box RBOX x 1
  float qlim[FSG_STENCIL_NOUT][2];  // planes' code bounds (q_min, q_max) as float32
};

// Device-side failures the host reads with fsg_kernel_errors (bit 0: a streaming-pass
// wait on a tensor copy ran out of polls).
__device__ unsigned g_kernel_errors;

// Fix-up list entry = unit | quarter << 28 | flags.  FIX_BAND: the quarter holds
// pixels within the stencil's reach of the window edge (np.gradient's one-sided
// formulas there); the fix-up recomputes those and the pixels whose stencil holds
// NoData.  No flag: only the latter.
constexpr unsigned FIX_BAND = 0x40000000u, FIX_QSHIFT = 28, FIX_UNIT = (1u << FIX_QSHIFT) - 1u;
// queue the quarters of unit u whose bit is set in qmask
__device__ __forceinline__ void push_fix(const FastArgs& A, int u, unsigned flags, unsigned qmask) {
  const unsigned n = __popc(qmask);
  unsigned i = atomicAdd(A.fix_count, n);
  for (unsigned q = 0; q < NQ; ++q)
    if ((qmask >> q) & 1u) A.fix_list[i++] = (unsigned)u | (q << FIX_QSHIFT) | flags;
}


// Unit geometry shared by the fast pass and the fix-up pass.
struct UnitGeom {
  int t, x0, y0, y1, xo;
};
__device__ __forceinline__ UnitGeom unit_geom(const FastArgs& A, int u) {
  int lo = 0, hi = A.ntiles - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (A.tiles[mid].unit0 <= u) lo = mid; else hi = mid - 1;
  }
  const FastTile& T = A.tiles[lo];
  const int lu = u - T.unit0;
  const int cy = lu / T.nstrip, sx = lu - (lu / T.nstrip) * T.nstrip;
  UnitGeom g;
  g.t = lo;
  g.x0 = T.cx0 + sx * SW;  // the last strip of a core may be narrower
  g.y0 = T.cy0 + cy * SH;
  g.y1 = min(g.y0 + SH, T.cy1);
  g.xo = min(g.x0 + SW, T.cx1);
  return g;
}

__device__ __forceinline__ void store_pixel(const FastArgs& A, unsigned om, bool allf32, char* const* optr,
                                            const float* o) {
#pragma unroll
  for (int kk = 0; kk < FSG_STENCIL_NOUT; ++kk) {
    if (!(om & (1u << kk))) continue;
    const PlaneK& P = A.planes[kk];
    char* dst = optr[kk];
    if (allf32 || P.dtype == FSG_F32) *reinterpret_cast<float*>(dst) = o[kk];
    else if (P.dtype == FSG_U8) *reinterpret_cast<uint8_t*>(dst) = (uint8_t)(int)quantize(o[kk], P.qa, P.qb, P.qmin, P.qmax);
    else *reinterpret_cast<int16_t*>(dst) = (int16_t)(int)quantize(o[kk], P.qa, P.qb, P.qmin, P.qmax);
  }
}

// Paired FP32 helpers (float2 = the two columns of a lane).
typedef float2 f2;
__device__ __forceinline__ f2 P2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ f2 S2(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
// Sums and differences on each component with the scalar _rn intrinsics, which are
// never contracted: for NumPy's float32 order where terms cancel (z * f[y+1] -
// z * f[y-1], the curvature and hillshade numerators, the quantiser's a * v + b).  A
// paired multiply followed by a paired difference was measured to give the
// once-rounded (fused) result there, even written as PTX mul.rn.f32x2 / sub.rn.f32x2;
// a paired product consumed by these scalar sums stays rounded.
__device__ __forceinline__ f2 nadd2(f2 a, f2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ f2 nsub2(f2 a, f2 b) { return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
// quantize_bits on a pair (the multiply, add and rounding add paired)
__device__ __forceinline__ uint2 quantize_bits2(f2 v, float qa, float qb, float fmin, float fmax) {
  f2 x = nadd2(mul2(v, S2(qa)), S2(qb));
  x.x = isfinite(v.x) ? fminf(fmaxf(x.x, fmin), fmax) : 0.0f;
  x.y = isfinite(v.y) ? fminf(fmaxf(x.y, fmin), fmax) : 0.0f;
  const f2 t = add2(x, S2(12582912.0f));
  return make_uint2(__float_as_uint(t.x), __float_as_uint(t.y));
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ bool nan2(f2 a) { return (a.x != a.x) | (a.y != a.y); }
// div_by on both components (Markstein's correction, as div_by)
__device__ __forceinline__ f2 div_by2(f2 a, float d, float r) {
  const f2 q = mul2(a, S2(r));
  const f2 e = fma2(q, S2(-d), a);  // q * -d == -(q * d) exactly
  return fma2(e, S2(r), q);
}
// arctan in degrees of a non-negative x: 6-term odd polynomial in a = min(x, 1/x)
// fitted (Lawson's iteratively reweighted least squares on Chebyshev nodes) to
// degrees(atan(a)) on [0, 1], |error| <= 1.1e-4 degree, and 90 - atan(1/x) above 1.
__device__ __forceinline__ f2 atan_deg_pos2(f2 x) {
  const bool i0 = x.x > 1.0f, i1 = x.y > 1.0f;
  const f2 a = P2(i0 ? rcp_approx(x.x) : x.x, i1 ? rcp_approx(x.y) : x.y);
  const f2 a2 = mul2(a, a);
  f2 p = S2(-0x1.57c936p-1f);
  p = fma2(a2, p, S2(0x1.821bb8p+1f));
  p = fma2(a2, p, S2(-0x1.aaed80p+2f));
  p = fma2(a2, p, S2(0x1.62d978p+3f));
  p = fma2(a2, p, S2(-0x1.30ed18p+4f));
  p = fma2(a2, p, S2(0x1.ca5b16p+5f));
  f2 r = mul2(a, p);
  r.x = i0 ? 90.0f - r.x : r.x;
  r.y = i1 ? 90.0f - r.y : r.y;
  return r;
}

// pixel_products for two pixels at once.  slx = sign_x * lx and sly =
// sign_y * ly (exact: the signs are +-1).  zone: pz, qz are p, q (z factor 1),
// so 1 + pz^2 + qz^2 is curvature's 1 + p^2 + q^2 and one rsqrt serves both.
// Curvature displays use t = -288.54 k = num / (den / 288.54), the constant
// folded into the denominators.
__device__ __forceinline__ void pixel_products2(const Light& L, float slx, float sly, bool zone, unsigned om, f2 p,
                                                f2 q, f2 pz, f2 qz, f2 dxx, f2 dxy, f2 dyy, f2 dyx, f2* o) {
  constexpr unsigned CURVM = (1u << FSG_OUT_CURV_MEAN) | (1u << FSG_OUT_CURV_GAUSSIAN) |
                             (1u << FSG_OUT_CURV_PLANFORM) | (1u << FSG_OUT_CURV_PROFILE);
  const f2 g2 = fma2(p, p, mul2(q, q));
  const f2 one_g2 = add2(S2(1.0f), g2);
  f2 rs1 = S2(0.f);  // rsqrt(1 + p^2 + q^2), when the hillshade computed it
  if (om & (1u << FSG_OUT_HILLSHADE)) {
    // the reference forms the numerator in float64 (its light vector is a float64
    // scalar): two fused multiply-adds stay closer to that than four roundings
    const f2 t = fma2(pz, S2(-slx), fma2(qz, S2(-sly), S2(L.lz)));
    const f2 n2 = zone ? one_g2 : add2(add2(mul2(pz, pz), mul2(qz, qz)), S2(1.0f));
    const f2 rs = P2(rsqrt_approx(n2.x), rsqrt_approx(n2.y));
    rs1 = rs;
    o[FSG_OUT_HILLSHADE] = P2(__saturatef(t.x * rs.x), __saturatef(t.y * rs.y));
  }
  if (om & (1u << FSG_OUT_SLOPE)) {
    if (L.slope_unit == FSG_SLOPE_DEGREE) {
      o[FSG_OUT_SLOPE] = atan_deg_pos2(P2(sqrt_approx(g2.x), sqrt_approx(g2.y)));
    } else {
      o[FSG_OUT_SLOPE] = P2(slope_value(p.x, q.x, L.slope_unit), slope_value(p.y, q.y, L.slope_unit));
    }
  }
  if (om & CURVM) {
    constexpr float C = 1.0f / 288.53900817779268f;  // den / 288.54: t = num / den'
    const f2 p2 = mul2(p, p), q2 = mul2(q, q), pq = mul2(p, q);
    // (1 + p^2 + q^2)^1.5
    const f2 sq1 = (zone && (om & (1u << FSG_OUT_HILLSHADE))) ? mul2(one_g2, rs1)
                                                              : P2(sqrt_approx(one_g2.x), sqrt_approx(one_g2.y));
    const f2 s15 = mul2(one_g2, sq1);
    const f2 pq2 = mul2(S2(2.0f), pq);
    const f2 g2c = mul2(g2, S2(C));
    auto display = [](f2 num, f2 den) {  // ((tanh(100k) + 1) / 2)^(1/2.2), k = -num / (288.54 den)
      const f2 t = mul2(num, P2(rcp_approx(den.x), rcp_approx(den.y)));
      const f2 e = P2(ex2_approx(t.x), ex2_approx(t.y));
      const f2 l = add2(S2(1.0f), e);
      const f2 m = mul2(S2(-0.45454545454545453f), P2(lg2_approx(l.x), lg2_approx(l.y)));
      return P2(ex2_approx(m.x), ex2_approx(m.y));
    };
    // Numerators in NumPy's float32 order, every operation rounded (no FMA): their
    // terms cancel on smooth terrain, so another rounding order moves k visibly.
    if (om & (1u << FSG_OUT_CURV_MEAN)) {
      const f2 sm = mul2(add2(dxy, dyx), S2(0.5f));
      const f2 num = nadd2(nsub2(mul2(nadd2(S2(1.0f), q2), dxx), mul2(pq2, sm)), mul2(nadd2(S2(1.0f), p2), dyy));
      o[FSG_OUT_CURV_MEAN] = display(num, fma2(S2(2.0f * C), s15, S2(1e-10f * C)));
    }
    if (om & (1u << FSG_OUT_CURV_GAUSSIAN)) {
      const f2 num = nsub2(mul2(dxx, dyy), mul2(dxy, dxy));
      const f2 den = mul2(one_g2, one_g2);
      o[FSG_OUT_CURV_GAUSSIAN] = display(P2(-num.x, -num.y), mul2(den, S2(C)));
    }
    if (om & (1u << FSG_OUT_CURV_PLANFORM)) {
      const f2 num = nadd2(nsub2(mul2(q2, dxx), mul2(pq2, dxy)), mul2(p2, dyy));
      o[FSG_OUT_CURV_PLANFORM] = display(num, fma2(g2c, P2(sqrt_approx(g2.x), sqrt_approx(g2.y)), S2(1e-10f * C)));
    }
    if (om & (1u << FSG_OUT_CURV_PROFILE)) {
      const f2 num = nadd2(nadd2(mul2(p2, dxx), mul2(pq2, dxy)), mul2(q2, dyy));
      o[FSG_OUT_CURV_PROFILE] = display(num, fma2(g2c, s15, S2(1e-10f * C)));
    }
  }
  o[FSG_OUT_DX] = p;
  o[FSG_OUT_DY] = q;
}

// Fast streaming pass (see above).  A warp owns a unit of SW = 128 columns and
// SH = 64 rows; lane l holds columns x0+4l .. x0+4l+3 as two float2 pairs, so
// every plane is written with one 16-byte store per lane (a 512-byte
// contiguous row segment per warp).  Rows reach the warp through a ring of RING
// rows in shared memory filled by cp.async (16 bytes per lane and row, plus the
// four halo columns x0-2, x0-1, x0+128, x0+129 copied by lane 0), RING-1 rows
// in flight.  Horizontal neighbours come from one shuffle each way per row and
// quantity; lanes 0 and 31 take theirs from the halo columns.  A warp vote per
// row tells whether any NoData lies in the rows feeding that output row; only
// then are the per-pixel checks evaluated.  DIV: derivatives use the correctly
// rounded division (bit-exact np.gradient, needed for the dx/dy planes);
// otherwise a multiply by the reciprocal.
#ifndef FSG_FAST_RING
#define FSG_FAST_RING 11  // rows per warp ring (RING - 1 copies in flight; 8 x 11 x 528 B static)
#endif
#ifndef FSG_FAST_MINB
#define FSG_FAST_MINB 2  // resident blocks per SM the register budget must allow
#endif
#ifndef FSG_FAST_NT
#define FSG_FAST_NT 256  // threads per block of the streaming pass (one unit per warp)
#endif
constexpr int RING = FSG_FAST_RING;
#ifndef FSG_FAST_ROW_UNROLL
#define FSG_FAST_ROW_UNROLL 1  // output rows per loop body (register renaming instead of moves)
#endif
constexpr int ROW_UNROLL = FSG_FAST_ROW_UNROLL;

__device__ __forceinline__ void cp_async16(unsigned dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(unsigned dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1; }" ::"r"(bar), "r"(bytes)
               : "memory");
}
// bounded wait for phase `parity` of the barrier: false when it did not complete in time
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    if (done) return true;
  }
  return false;
}
// one box of the 2-D tensor map at element (x, y) into shared memory, completion on `bar`
__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap* map, int x, int y, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Four columns of a lane as two pairs, plus the lane's edge pair: lane 0 keeps
// (f[x0-2], f[x0-1]) and lane 31 (f[x0+128], f[x0+129]) (unused elsewhere).
struct Q4 {
  f2 lo, hi;
};
__device__ __forceinline__ Q4 q4add(Q4 a, Q4 b) { return {add2(a.lo, b.lo), add2(a.hi, b.hi)}; }
__device__ __forceinline__ Q4 q4sub(Q4 a, Q4 b) { return {sub2(a.lo, b.lo), sub2(a.hi, b.hi)}; }
// f(c+1) - f(c-1) for the four columns, left = f(x-1), right = f(x+4)
__device__ __forceinline__ Q4 q4hdiff(Q4 f, float left, float right) {
  return {sub2(P2(f.lo.y, f.hi.x), P2(left, f.lo.x)), sub2(P2(f.hi.y, right), P2(f.lo.y, f.hi.x))};
}

// ZONE: z factor 1 (hillshade's derivatives are p, q; rows above/below the
// stencil's own window are then never read again, so they are not kept).
// PK: the planes' types, 1 all float32, 2 all uint8 (each without runtime type tests),
// 0 any mix (tested per plane).
template <bool CURV, unsigned OM, int PK, bool ZONE>
__global__ void __launch_bounds__(FSG_FAST_NT, FSG_FAST_MINB) stencil_fast_kernel(const __grid_constant__ FastArgs A) {
  constexpr bool ALLF32 = PK == 1, ALLU8 = PK == 2;
  constexpr bool DIV = (OM & ((1u << FSG_OUT_DX) | (1u << FSG_OUT_DY))) != 0;
  constexpr int REACH = CURV ? 2 : 1;  // rows above / below an output row that feed it
  extern __shared__ __align__(1024) float ring_dyn[];  // [warps][RING][RW] floats, then [warps][RING] barriers
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  float* ring = ring_dyn + (size_t)(threadIdx.x >> 5) * RING * RW;
  const unsigned sbase = (unsigned)__cvta_generic_to_shared(ring);
  const unsigned bbase = (unsigned)__cvta_generic_to_shared(ring_dyn + (size_t)(FSG_FAST_NT / 32) * RING * RW) +
                         (unsigned)(threadIdx.x >> 5) * RING * 8u;  // this warp's RING barriers
  if (A.use_tma) {
    if (lane == 0) {
      for (int i = 0; i < RING; ++i) mbar_init(bbase + 8u * i, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncwarp();
  }
  unsigned tma_issued = 0, tma_taken = 0;  // rows of this warp through the tensor path (slot, phase)
  const bool hn = A.has_nodata != 0;
  const Light L{A.lx, A.ly, A.lz, A.slope_unit};
  const float qnan = __int_as_float(0x7fc00000);
  const bool e0lane = lane == 0, e31lane = lane == 31;
  // Units of all tiles (of any size and overview level) are popped from one device
  // queue, one per warp at a time, so warps that draw cheap units take more of them.
  auto pop = [&]() -> int {
    unsigned v = 0;
    if (lane == 0) v = atomicAdd(A.queue, 1u);
    return (int)__shfl_sync(0xffffffffu, v, 0);
  };
  (void)warp;
  (void)nwarps;
  for (int u = pop(); u < A.total_units; u = pop()) {
    const UnitGeom g = unit_geom(A, u);
    const FastTile& TG = A.tiles[g.t];
    const int x0 = g.x0, y0 = g.y0, y1 = g.y1, xo = g.xo;
    // stencil reach: rows y0-2 .. y1+1 and cols x0-2 .. xo+1 strictly inside
    // the window, so every derivative is a central difference
    const bool interior = y0 - 2 >= TG.wy0 && y1 + 2 <= TG.wy1 && x0 - 2 >= TG.wx0 && xo + 2 <= TG.wx1;
    // A unit at the window edge runs here too: the rows and columns its stencil takes
    // from beyond the window (zeros from the tensor copy outside the raster, stale ring
    // rows on the cp.async path, which copies nothing outside the window) reach only
    // the pixels within the stencil's reach of the edge, which the fix-up recomputes.
    // the tile's constants as values: the plane stores below could alias the
    // tile table as far as the compiler knows, which would force reloads
    struct Step {
      float d2, rcp;
    };
    struct {
      Step g1x, g1y, c2x, c2y;
      float slx, sly;
      int oy0, ox0, cy0, cx0, wx1;
    } const T = {{TG.g1x.d2, TG.g1x.rcp}, {TG.g1y.d2, TG.g1y.rcp}, {TG.c2x.d2, TG.c2x.rcp},
                 {TG.c2y.d2, TG.c2y.rcp}, TG.sx * L.lx, TG.sy * L.ly, TG.oy0, TG.ox0, TG.cy0, TG.cx0, TG.wx1};
    const int xl = x0 + 4 * lane;  // first column of this lane
    // output columns of this lane: xl + m < xo
    const int nout = min(4, max(0, xo - xl));
    // 16-byte copies need a 16-byte aligned start for every row (uniform per unit)
    const bool vload = ((A.ld & 3) == 0) && ((((uintptr_t)A.raster >> 2) + (uintptr_t)x0) & 3) == 0;
    // the tensor path: one box per row from x0-4, whose x must be a multiple of 4 elements
    const bool tma = A.use_tma && (x0 & 3) == 0;
    const bool lfull = xl + 3 < T.wx1;
    const int nrows = (y1 - y0) + 2 * REACH;      // rows y0-REACH .. y1+REACH-1
    const float* src0 = A.raster + (long long)(y0 - REACH) * A.ld;
    const unsigned tma0 = tma_issued;             // this unit's first tensor-path row
    bool failed = false;
    if (tma && lane == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // after any cp.async unit
    __syncwarp();
    // row k of the unit -> ring slot; RING-1 rows in flight
    auto issue = [&](int k) {
      if (tma) {
        if (k < nrows) {
          const unsigned slot = (tma0 + (unsigned)k) % RING;
          if (lane == 0) {
            mbar_expect_tx(bbase + 8u * slot, RBOX * 4);
            tma_load_2d(sbase + slot * (RW * 4), &A.tmap, x0 - 4, y0 - REACH + k, bbase + 8u * slot);
          }
          ++tma_issued;
        }
        return;
      }
      const int ry = y0 - REACH + k;
      if (k < nrows && ry >= TG.wy0 && ry < TG.wy1) {  // rows of the window only
        const float* gp = src0 + (long long)k * A.ld;
        const unsigned dst = sbase + (unsigned)((k % RING) * (RW * 4));
        if (vload && lfull) {
          cp_async16(dst + 16 + 16 * lane, gp + xl);
        } else {
#pragma unroll
          for (int m = 0; m < 4; ++m)
            if (xl + m < T.wx1) cp_async4(dst + 16 + 4 * (4 * lane + m), gp + xl + m);
        }
        if (lane == 0) {
          if (x0 - 2 >= TG.wx0) {
            cp_async4(dst + 8, gp + x0 - 2);
            cp_async4(dst + 12, gp + x0 - 1);
          }
          if (x0 + SW + 1 < T.wx1) {
            cp_async4(dst + 4 * (SW + 4), gp + x0 + SW);
            cp_async4(dst + 4 * (SW + 5), gp + x0 + SW + 1);
          }
        }
      }
      cp_async_commit();
    };
    int nan_left = 0;  // rows for which the NoData seen last still feeds an output
    // take row k: the lane's four columns and its edge pair
    auto take = [&](int k, Q4& f, f2& e) {
      const float* rp;
      if (tma) {
        const unsigned slot = tma_taken % RING, parity = (tma_taken / RING) & 1u;
        if (!mbar_wait(bbase + 8u * slot, parity)) failed = true;
        ++tma_taken;
        rp = ring + slot * RW;
      } else {
        cp_async_wait<RING - 2>();
        __syncwarp();
        rp = ring + (k % RING) * RW;
      }
      const float4 v = *reinterpret_cast<const float4*>(rp + 4 + 4 * lane);
      const float2 h = *reinterpret_cast<const float2*>(rp + (e31lane ? SW + 4 : 2));
      f = {P2(v.x, v.y), P2(v.z, v.w)};
      e = P2(h.x, h.y);
      __syncwarp();
      issue(k + RING - 1);
      if (hn) {
        if (is_nodata(f.lo.x, A.ndf, true)) f.lo.x = qnan;
        if (is_nodata(f.lo.y, A.ndf, true)) f.lo.y = qnan;
        if (is_nodata(f.hi.x, A.ndf, true)) f.hi.x = qnan;
        if (is_nodata(f.hi.y, A.ndf, true)) f.hi.y = qnan;
        if (is_nodata(e.x, A.ndf, true)) e.x = qnan;
        if (is_nodata(e.y, A.ndf, true)) e.y = qnan;
      }
      if (nan2(f.lo) || nan2(f.hi) || ((e0lane || e31lane) && nan2(e))) nan_left = 2 * REACH + 1;
    };
#pragma unroll 1
    for (int k = 0; k < RING - 1; ++k) issue(k);
    // by value: a reference would give the steps an address (a stack slot and a local load per use)
    auto dv = [](f2 num, Step a) { return DIV ? div_by2(num, a.d2, a.rcp) : mul2(num, S2(a.rcp)); };
    auto dv4 = [&](Q4 num, Step a) { return Q4{dv(num.lo, a), dv(num.hi, a)}; };
    auto dv1 = [](float num, Step a) { return DIV ? div_by(num, a.d2, a.rcp) : __fmul_rn(num, a.rcp); };
    // The curvature's derivatives are always correctly rounded: the second differences of
    // np.gradient's float32 first derivatives amplify a one-ulp difference in them (by
    // ~|dx| / |dxx step|, up to ~1e3 on smooth terrain), and the numerators cancel.
    auto dv4e = [](Q4 num, Step a) { return Q4{div_by2(num.lo, a.d2, a.rcp), div_by2(num.hi, a.d2, a.rcp)}; };
    auto dv1e = [](float num, Step a) { return div_by(num, a.d2, a.rcp); };
    // horizontal central difference of a row: neighbours from the adjacent lanes or the edge pair
    auto hdiff = [&](Q4 f, f2 e) {
      float left = __shfl_up_sync(0xffffffffu, f.hi.y, 1), right = __shfl_down_sync(0xffffffffu, f.lo.x, 1);
      if (e0lane) left = e.y;   // f[x0-1]
      if (e31lane) right = e.x; // f[x0+128]
      return q4hdiff(f, left, right);
    };
    // the edge lanes' derivative one column outside the unit: lane 0 at x0-1, lane 31 at x0+128
    auto edge_dx = [&](Q4 f, f2 e) { return e31lane ? __fsub_rn(e.y, f.hi.y) : __fsub_rn(f.lo.x, e.x); };
    char* optr[FSG_STENCIL_NOUT];
    long long ostep[FSG_STENCIL_NOUT];
    bool vstore[FSG_STENCIL_NOUT];
#pragma unroll
    for (int k = 0; k < FSG_STENCIL_NOUT; ++k) {
      if (!(OM & (1u << k))) continue;
      const PlaneK& P = A.planes[k];
      const int esz = ALLF32 ? 4 : ALLU8 ? 1 : (P.dtype == FSG_F32 ? 4 : (P.dtype == FSG_I16 ? 2 : 1));
      const long long col = (long long)(T.ox0 + xl - T.cx0);
      optr[k] = static_cast<char*>(P.ptr) + ((long long)(T.oy0 + y0 - T.cy0) * P.ld + col) * esz;
      ostep[k] = P.ld * esz;
      // four pixels of a lane in one store: 16 bytes (float32), 8 (int16) or 4 (uint8) at an
      // address aligned to that size (the row pitch and the unit's first column keep it)
      const uintptr_t a0 = (uintptr_t)P.ptr + (uintptr_t)((long long)(T.ox0 + x0 - T.cx0) * esz);
      vstore[k] = ((P.ld & 3) == 0) && (a0 % (uintptr_t)(4 * esz)) == 0;
    }
    int kr = 0;  // next unit row to take
    Q4 fm2{}, fm1, f0, fp1, fp2{};
    f2 em2 = S2(0.f), em1, e0, ep1, ep2 = S2(0.f);
    if (CURV) take(kr++, fm2, em2);
    take(kr++, fm1, em1);
    take(kr++, f0, e0);
    take(kr++, fp1, ep1);
    if (CURV) take(kr++, fp2, ep2);
    // first derivatives of rows -1 and 0 (curvature), with the edge lanes' outside column
    Q4 dxm1{}, dym1{}, dx0{}, dy0{};
    float xd0 = 0.f, yd0 = 0.f;  // edge-lane dx / dy of row 0 (outside column)
    if (CURV) {
      dxm1 = dv4e(hdiff(fm1, em1), T.g1x);
      dym1 = dv4e(q4sub(f0, fm2), T.g1y);
      dx0 = dv4e(hdiff(f0, e0), T.g1x);
      dy0 = dv4e(q4sub(fp1, fm1), T.g1y);
      xd0 = dv1e(edge_dx(f0, e0), T.g1x);
      yd0 = dv1e(__fsub_rn(e31lane ? ep1.x : ep1.y, e31lane ? em1.x : em1.y), T.g1y);
    }
    bool bad = false;
#pragma unroll ROW_UNROLL
    for (int y = y0; y < y1; ++y) {
      // NoData in the 2*REACH+1 rows feeding this output row (any lane)?
      const bool row_nan = __any_sync(0xffffffffu, nan_left > 0);
      Q4 p, q, dxx{}, dxy{}, dyy{}, dyx{}, dxp1{}, dyp1{};
      float xp1 = 0.f, yp1 = 0.f;
      if (CURV) {
        dxp1 = dv4e(hdiff(fp1, ep1), T.g1x);
        dyp1 = dv4e(q4sub(fp2, f0), T.g1y);
        xp1 = dv1e(edge_dx(fp1, ep1), T.g1x);
        yp1 = dv1e(__fsub_rn(e31lane ? ep2.x : ep2.y, e31lane ? e0.x : e0.y), T.g1y);
        p = dx0;
        q = dy0;
        dxx = dv4e(hdiff(dx0, P2(xd0, xd0)), T.c2x);
        dxy = dv4e(q4sub(dxp1, dxm1), T.c2y);
        dyy = dv4e(q4sub(dyp1, dym1), T.c2y);
        if (OM & (1u << FSG_OUT_CURV_MEAN)) dyx = dv4e(hdiff(dy0, P2(yd0, yd0)), T.c2x);
      } else {
        p = dv4(hdiff(f0, e0), T.g1x);
        q = dv4(q4sub(fp1, fm1), T.g1y);
      }
      Q4 pz = p, qz = q;
      if ((OM & (1u << FSG_OUT_HILLSHADE)) && !ZONE) {
        const f2 zf = S2(A.z);
        // z * f rounded before the difference, as NumPy's (dem * z) then np.gradient
        auto zq = [&](Q4 f) { return Q4{mul2(f.lo, zf), mul2(f.hi, zf)}; };
        const Q4 zc = zq(f0);
        const f2 ze = mul2(e0, zf);
        float left = __shfl_up_sync(0xffffffffu, zc.hi.y, 1), right = __shfl_down_sync(0xffffffffu, zc.lo.x, 1);
        if (e0lane) left = ze.y;
        if (e31lane) right = ze.x;
        pz = dv4(Q4{nsub2(P2(zc.lo.y, zc.hi.x), P2(left, zc.lo.x)), nsub2(P2(zc.hi.y, right), P2(zc.lo.y, zc.hi.x))},
                 T.g1x);
        const Q4 zp = zq(fp1), zm = zq(fm1);
        qz = dv4(Q4{nsub2(zp.lo, zm.lo), nsub2(zp.hi, zm.hi)}, T.g1y);
      }
      if (row_nan) {
        Q4 chk = q4add(p, q);
        if ((OM & (1u << FSG_OUT_HILLSHADE)) && !ZONE) chk = q4add(chk, q4add(pz, qz));
        if (CURV) chk = q4add(q4add(chk, q4add(dxx, dxy)), q4add(dyy, dyx));
        bad |= (nout > 0 && f0.lo.x == f0.lo.x && chk.lo.x != chk.lo.x) ||
               (nout > 1 && f0.lo.y == f0.lo.y && chk.lo.y != chk.lo.y) ||
               (nout > 2 && f0.hi.x == f0.hi.x && chk.hi.x != chk.hi.x) ||
               (nout > 3 && f0.hi.y == f0.hi.y && chk.hi.y != chk.hi.y);
      }
      f2 olo[FSG_STENCIL_NOUT], ohi[FSG_STENCIL_NOUT];
      pixel_products2(L, T.slx, T.sly, ZONE, OM, p.lo, q.lo, pz.lo, qz.lo, dxx.lo, dxy.lo, dyy.lo,
                      dyx.lo, olo);
      pixel_products2(L, T.slx, T.sly, ZONE, OM, p.hi, q.hi, pz.hi, qz.hi, dxx.hi, dxy.hi, dyy.hi,
                      dyx.hi, ohi);
      if (nan2(f0.lo) || nan2(f0.hi)) {
#pragma unroll
        for (int kk = 0; kk < FSG_STENCIL_NOUT; ++kk) {
          if (f0.lo.x != f0.lo.x) olo[kk].x = qnan;
          if (f0.lo.y != f0.lo.y) olo[kk].y = qnan;
          if (f0.hi.x != f0.hi.x) ohi[kk].x = qnan;
          if (f0.hi.y != f0.hi.y) ohi[kk].y = qnan;
        }
      }
#pragma unroll
      for (int kk = 0; kk < FSG_STENCIL_NOUT; ++kk) {
        if (!(OM & (1u << kk))) continue;
        char* dst = optr[kk];
        if (ALLF32 || (!ALLU8 && A.planes[kk].dtype == FSG_F32)) {
          if (vstore[kk] && nout == 4) {
            *reinterpret_cast<float4*>(dst) = make_float4(olo[kk].x, olo[kk].y, ohi[kk].x, ohi[kk].y);
          } else {
            float* d = reinterpret_cast<float*>(dst);
            if (nout > 0) d[0] = olo[kk].x;
            if (nout > 1) d[1] = olo[kk].y;
            if (nout > 2) d[2] = ohi[kk].x;
            if (nout > 3) d[3] = ohi[kk].y;
          }
        } else {
          // code bit patterns (quantize_bits: the code in the low 8 / 16 bits)
          const PlaneK& P = A.planes[kk];
          const float fmin = A.qlim[kk][0], fmax = A.qlim[kk][1];
          const uint2 cl = quantize_bits2(olo[kk], P.qa, P.qb, fmin, fmax);
          const uint2 ch = quantize_bits2(ohi[kk], P.qa, P.qb, fmin, fmax);
          const uint32_t c[4] = {cl.x, cl.y, ch.x, ch.y};
          if (ALLU8 || P.dtype == FSG_U8) {
            if (vstore[kk] && nout == 4) {  // one 4-byte store: a warp writes 128 contiguous bytes
              *reinterpret_cast<uint32_t*>(dst) =
                  __byte_perm(__byte_perm(c[0], c[1], 0x0040), __byte_perm(c[2], c[3], 0x0040), 0x5410);
            } else {
#pragma unroll
              for (int m = 0; m < 4; ++m)
                if (m < nout) reinterpret_cast<uint8_t*>(dst)[m] = (uint8_t)c[m];
            }
          } else {
            if (vstore[kk] && nout == 4) {  // one 8-byte store
              *reinterpret_cast<uint2*>(dst) = make_uint2(__byte_perm(c[0], c[1], 0x5410), __byte_perm(c[2], c[3], 0x5410));
            } else {
#pragma unroll
              for (int m = 0; m < 4; ++m)
                if (m < nout) reinterpret_cast<uint16_t*>(dst)[m] = (uint16_t)c[m];
            }
          }
        }
        optr[kk] += ostep[kk];
      }
      // slide one row down
      if (nan_left > 0) --nan_left;
      if (y + 1 < y1) {
        Q4 nx;
        f2 ne;
        take(kr++, nx, ne);
        if (CURV) {
          fm2 = fm1; fm1 = f0; f0 = fp1; fp1 = fp2; fp2 = nx;
          em2 = em1; em1 = e0; e0 = ep1; ep1 = ep2; ep2 = ne;
          dxm1 = dx0; dym1 = dy0; dx0 = dxp1; dy0 = dyp1;
          xd0 = xp1; yd0 = yp1;
        } else {
          fm1 = f0; f0 = fp1; fp1 = nx;
          em1 = e0; e0 = ep1; ep1 = ne;
        }
      }
    }
    if (tma && __any_sync(0xffffffffu, failed)) {
      // a tensor copy did not arrive in time: record it, give the copies still in flight a
      // bounded wait, and stop this warp (the host reads the flag with fsg_kernel_errors)
      if (lane == 0) {
        atomicOr(&g_kernel_errors, 1u);
        for (unsigned r = tma_taken; r < tma_issued; ++r) mbar_wait(bbase + 8u * (r % RING), (r / RING) & 1u);
      }
      __syncwarp();
      return;
    }
    // quarters (eight lanes each) holding a pixel whose stencil reached NoData, and at a
    // window edge the quarters holding pixels within the stencil's reach of it
    const unsigned bb = __ballot_sync(0xffffffffu, bad);
    if (lane == 0) {
      unsigned qm = 0, qb = 0;
      for (unsigned qq = 0; qq < NQ; ++qq) qm |= ((bb >> (8 * qq)) & 0xffu) ? (1u << qq) : 0u;
      if (!interior) {
        const bool rows_band = y0 < TG.wy0 + REACH || y1 > TG.wy1 - REACH;
        for (int qq = 0; qq < NQ; ++qq) {
          const int qx0 = x0 + qq * FW, qx1 = min(qx0 + FW, xo);
          if (qx0 < qx1 && (rows_band || qx0 < TG.wx0 + REACH || qx1 > TG.wx1 - REACH)) qb |= 1u << qq;
        }
      }
      if (qb) push_fix(A, u, FIX_BAND, qb);
      if (qm & ~qb) push_fix(A, u, 0u, qm & ~qb);
    }
  }
  cp_async_wait<0>();
}

// ------------------------------------------------------------- fix-up pass
// One CTA per listed quarter recomputes, with the full reference semantics in
// shared memory, its pixels whose stencil holds NoData or (FIX_BAND) reaches the
// window edge: NoData cells within reach of a valid
// output pixel get the NaN-aware Gaussian fill (_nan_utils.py:18-31: separable
// sigma = 1, radius 4, 'nearest' at the window edges, axis 0 then axis 1 with a
// float32 intermediate, sums in float-float), then np.gradient with the
// window's edge rules and the second derivatives on the signed steps.
// Regions, relative to the unit origin (y0, x0):
//   S  source values        rows -8 .. SH+8, cols -8 .. FW+8 (NaN outside the window)
//   E  filled values        rows -4 .. SH+4, cols -4 .. FW+4
//   D  first derivatives    rows -2 .. SH+2, cols -2 .. FW+2 (curvature only)
// for each quarter (FW columns) of the unit.
constexpr int XS_R = SH + 16, XS_C = FW + 16;  // 80 x 48
constexpr int XE_R = SH + 8, XE_C = FW + 8;    // 72 x 40
constexpr int XD_R = SH + 4, XD_C = FW + 4;    // 68 x 36
constexpr int XNT = 256;
constexpr int XL_ROWS = 96;  // row offsets of a compacted cell list (rows <= XS_R)
constexpr size_t FIX_SMEM = sizeof(float) * XS_R * XS_C +                  // source (filled in place)
                            sizeof(float) * 2 * XE_R * XS_C +            // axis-0 sums (aliases D)
                            sizeof(unsigned long long) * 5 * XE_R +       // row bitmasks
                            sizeof(int) * XL_ROWS +                       // compacted list: row offsets
                            sizeof(unsigned short) * XE_R * XS_C;         //   and (row << 8 | column) entries
static_assert(XS_R <= XL_ROWS - 1 && XS_C <= 64, "compacted list: 16-bit entries, one offset slot spare");
static_assert(XE_R <= 128 && 128 + XE_R <= XNT, "stage (c): one E row per thread in warps 0-3 and in warps 4-7");

static_assert(2 * XD_R * XD_C <= 2 * XE_R * XS_C, "derivative planes alias the axis-0 sums");
// the output list of stage (g) sits after the derivative planes, in the axis-0 sums' tail
constexpr int XG_OFF = 2 * XD_R * XD_C;
static_assert(XG_OFF + XL_ROWS + (SH * FW + 1) / 2 <= 2 * XE_R * XS_C, "output list in the sums' tail");
static_assert(XE_C <= 64 && XS_C <= 64, "row bitmasks are 64 bits");

template <bool DIV, class Fn>
__device__ __forceinline__ float deriv_d(const Axis& a, int k, int lo, int hi, Fn f) {
  if (k > lo && k < hi - 1) {
    const float num = fsub(f(1), f(-1));
    return DIV ? div_by(num, a.d2, a.rcp) : fmul(num, a.rcp);
  }
  if (k == lo) return fadd(fadd(fmul(a.fa, f(0)), fmul(a.fb, f(1))), fmul(a.fc, f(2)));
  return fadd(fadd(fmul(a.ba, f(-2)), fmul(a.bb, f(-1))), fmul(a.bc, f(0)));
}

template <unsigned OM, bool ALLF32>
__global__ void __launch_bounds__(XNT, 4) stencil_fixup_kernel(const __grid_constant__ FastArgs A) {
  constexpr bool CURV = (OM & ((1u << FSG_OUT_CURV_MEAN) | (1u << FSG_OUT_CURV_GAUSSIAN) |
                               (1u << FSG_OUT_CURV_PLANFORM) | (1u << FSG_OUT_CURV_PROFILE))) != 0;
  constexpr bool DIV = (OM & ((1u << FSG_OUT_DX) | (1u << FSG_OUT_DY))) != 0;
  extern __shared__ __align__(16) unsigned char fix_smem[];
  // the source region; the fills of stage (e) go in place, so its E part is the filled surface
  float* Sv = reinterpret_cast<float*>(fix_smem);
  float* VV = Sv + XS_R * XS_C;
  float* VW = VV + XE_R * XS_C;
  float* DX = VV;  // reused once the fills are done
  float* DY = DX + XD_R * XD_C;
  unsigned long long* VO = reinterpret_cast<unsigned long long*>(VW + XE_R * XS_C);  // valid output pixels
  unsigned long long* NB = VO + XE_R;   // NoData cells inside the window
  unsigned long long* ND = NB + XE_R;   // cells to fill (E columns)
  unsigned long long* NV = ND + XE_R;   // axis-0 sums to form (S columns)
  unsigned long long* AF = NV + XE_R;   // valid outputs whose stencil holds NoData (the fast pass's others stand)
  int* LOFF = reinterpret_cast<int*>(AF + XE_R);                      // [XL_ROWS] list row offsets, total last
  unsigned short* LST = reinterpret_cast<unsigned short*>(LOFF + XL_ROWS);  // [XE_R * XS_C] (row << 8 | column)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool hn = A.has_nodata != 0;
  const float qnan = __int_as_float(0x7fc00000);
  // The cells of a stage (set bits of its per-row masks) as one list, so that every
  // lane of a pass works on a cell that needs it: per-row counts scanned by one warp
  // (three rows per lane; the masks kept in `keep` when given), then each warp writes
  // its rows, each lane the entry of its column (position = the set bits below it).
  // compact is called by every thread (two barriers) and returns the number of cells.
  auto scan_rows = [&](int nrows, auto rowmask, int* loff, unsigned long long* keep) {
    int c3[3], sum = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int r = 3 * lane + j;
      unsigned long long m = 0;
      if (r < nrows) {
        m = rowmask(r);
        if (keep) keep[r] = m;
      }
      c3[j] = __popcll(m);
      sum += c3[j];
    }
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += n;
    }
    int base = incl - sum;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int r = 3 * lane + j;
      if (r < nrows) loff[r] = base;
      base += c3[j];
    }
    if (lane == 31) loff[XL_ROWS - 1] = incl;
  };
  auto write_rows = [&](int nrows, auto rowmask, const int* loff, unsigned short* lst) {
    for (int r = warp; r < nrows; r += XNT / 32) {
      const unsigned long long m = rowmask(r);
      const int o = loff[r];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int c = 32 * h + lane;
        if ((m >> c) & 1ull) lst[o + __popcll(m & ((1ull << c) - 1ull))] = (unsigned short)((r << 8) | c);
      }
    }
  };
  auto compact = [&](int nrows, const unsigned long long* rm) -> int {
    auto mk = [&](int r) { return rm[r]; };
    if (warp == 0) scan_rows(nrows, mk, LOFF, nullptr);
    __syncthreads();
    write_rows(nrows, mk, LOFF, LST);
    __syncthreads();
    return LOFF[XL_ROWS - 1];
  };
  const unsigned count = *A.fix_count;
  // listed quarters popped from a queue (their costs differ: NoData fills, edge bands);
  // the next entry is popped after the first barrier of the current one
  __shared__ unsigned s_it;
  if (tid == 0) s_it = atomicAdd(A.fix_queue, 1u);
  __syncthreads();
  for (;;) {
    const unsigned it = s_it;
    if (it >= count) break;
    const unsigned e = A.fix_list[it];
    const bool band = (e & FIX_BAND) != 0;
    const UnitGeom g = unit_geom(A, (int)(e & FIX_UNIT));
    const FastTile& T = A.tiles[g.t];
    const int x0 = g.x0 + (int)((e >> FIX_QSHIFT) & (NQ - 1)) * FW, y0 = g.y0, y1 = g.y1, xo = min(x0 + FW, g.xo);
    if (x0 >= xo) {  // (not listed by the streaming pass; kept safe)
      __syncthreads();
      if (tid == 0) s_it = atomicAdd(A.fix_queue, 1u);
      __syncthreads();
      continue;
    }
    // (a) source region: cells inside the window copied with cp.async (all in
    //     flight at once; four cells per 16-byte copy where the row allows), the
    //     rest NaN (never read); then NoData -> NaN
    {
      static_assert(XS_C % 4 == 0, "16-byte chunks of the source rows");
      const unsigned sv0 = (unsigned)__cvta_generic_to_shared(Sv);
      for (int q = tid; q < XS_R * (XS_C / 4); q += XNT) {
        const int r = q / (XS_C / 4), c = 4 * (q - r * (XS_C / 4)), i = r * XS_C + c;
        const int gy = y0 - 8 + r, gx = x0 - 8 + c;
        if (gy < T.wy0 || gy >= T.wy1) {
#pragma unroll
          for (int m = 0; m < 4; ++m) Sv[i + m] = qnan;
          continue;
        }
        const float* row = A.raster + (long long)gy * A.ld;
        if (gx >= T.wx0 && gx + 3 < T.wx1 && (reinterpret_cast<uintptr_t>(row + gx) & 15) == 0) {
          cp_async16(sv0 + 4u * (unsigned)i, row + gx);
        } else {
#pragma unroll
          for (int m = 0; m < 4; ++m) {
            if (gx + m >= T.wx0 && gx + m < T.wx1) cp_async4(sv0 + 4u * (unsigned)(i + m), row + gx + m);
            else Sv[i + m] = qnan;
          }
        }
      }
      cp_async_commit();
      cp_async_wait<0>();
      if (hn) {  // each thread its own copies (complete and visible to it after the wait)
        for (int q = tid; q < XS_R * (XS_C / 4); q += XNT) {
#pragma unroll
          for (int m = 0; m < 4; ++m)
            if (is_nodata(Sv[4 * q + m], A.ndf, true)) Sv[4 * q + m] = qnan;
        }
      }
      __syncthreads();
      if (tid == 0) s_it = atomicAdd(A.fix_queue, 1u);  // every thread has read this entry
    }
    // (b) row bitmasks of valid output pixels and of in-window NoData cells
    for (int r = warp; r < XE_R; r += XNT / 32) {
      const int gy = y0 - 4 + r;
      const bool row_out = gy >= y0 && gy < y1, row_win = gy >= T.wy0 && gy < T.wy1;
      unsigned long long vo = 0, nb = 0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int c = h * 32 + lane;
        bool o = false, n = false;
        if (c < XE_C) {
          const float v = Sv[(r + 4) * XS_C + c + 4];
          const int gx = x0 - 4 + c;
          o = row_out && gx >= x0 && gx < xo && v == v;
          n = row_win && gx >= T.wx0 && gx < T.wx1 && v != v;
        }
        vo |= (unsigned long long)__ballot_sync(0xffffffffu, o) << (32 * h);
        nb |= (unsigned long long)__ballot_sync(0xffffffffu, n) << (32 * h);
      }
      if (lane == 0) {
        VO[r] = vo;
        NB[r] = nb;
      }
    }
    __syncthreads();
    // (c) NoData cells within the derivative reach of a valid output pixel:
    //     2 for central differences, 3 where one-sided edge formulas occur
    const int R = band ? 3 : 2;
    bool any = false;
    if (tid < XE_R) {
      unsigned long long v = 0;
      for (int k = -R; k <= R; ++k)
        if (tid + k >= 0 && tid + k < XE_R) v |= VO[tid + k];
      unsigned long long d = v;
      for (int k = 1; k <= R; ++k) d |= (v << k) | (v >> k);
      const unsigned long long need = d & NB[tid];
      ND[tid] = need;
      any = need != 0;
      {  // axis-0 sums needed by the axis-1 pass: S columns within 4 of a cell to fill, inside the window
        const unsigned long long n = need << 4;
        unsigned long long dn = n;
#pragma unroll
        for (int k = 1; k <= 4; ++k) dn |= (n << k) | (n >> k);
        const int c_lo = max(T.wx0 - (x0 - 8), 0), c_hi = min(T.wx1 - (x0 - 8), XS_C);
        const unsigned long long win =
            c_hi > c_lo ? (((c_hi - c_lo) >= 64 ? ~0ull : ((1ull << (c_hi - c_lo)) - 1ull)) << c_lo) : 0ull;
        NV[tid] = dn & win;
      }
    } else if (tid >= 128 && tid < 128 + XE_R) {  // (other warps) the outputs to recompute
      const int er = tid - 128;
      // outputs whose stencil footprint (a (2K+1)^2 box) contains a NoData cell
      constexpr int K = CURV ? 2 : 1;
      unsigned long long nbr = 0;
      for (int k = -K; k <= K; ++k)
        if (er + k >= 0 && er + k < XE_R) nbr |= NB[er + k];
      unsigned long long dil = nbr;
      for (int k = 1; k <= K; ++k) dil |= (nbr << k) | (nbr >> k);
      unsigned long long af = VO[er] & dil;
      if (band) {  // the valid pixels within the stencil's reach of the window edge
        constexpr int EB = CURV ? 2 : 1;
        const int gy = y0 - 4 + er;
        unsigned long long bm = 0;
        if (gy < T.wy0 + EB || gy >= T.wy1 - EB) {
          bm = ~0ull;
        } else {
          auto cols = [](int a, int b) {  // E columns [a, b) clipped to [0, 64)
            a = max(a, 0);
            b = min(b, 64);
            return a >= b ? 0ull : ((b - a >= 64 ? ~0ull : ((1ull << (b - a)) - 1ull)) << a);
          };
          const int l0 = T.wx0 - (x0 - 4), h1 = T.wx1 - (x0 - 4);
          bm = cols(l0, l0 + EB) | cols(h1 - EB, h1);
        }
        af |= VO[er] & bm;
      }
      AF[er] = af;
    }
    if (__syncthreads_or(any)) {
      // (d) axis-0 sums of the S cells listed in NV
      FF gw[5];
#pragma unroll
      for (int j = 0; j < 5; ++j) gw[j] = A.gw[j];
      const int nv = compact(XE_R, NV);
      for (int li = tid; li < nv; li += XNT) {
        const int r = LST[li] >> 8, sc = LST[li] & 255, i = r * XS_C + sc;
        const int gy = y0 - 4 + r;
        float xv[9], xw[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int yy = min(max(gy + j - 4, T.wy0), T.wy1 - 1);
          const float v = Sv[(yy - (y0 - 8)) * XS_C + sc];
          const bool ok = v == v;
          xv[j] = ok ? v : 0.f;
          xw[j] = ok ? 1.f : 0.f;
        }
        const float2 sw2 = gsum_ff2(gw, xv, xw);
        VV[i] = sw2.x;
        VW[i] = sw2.y;
      }
      __syncthreads();
      // (e) axis-1 pass and the normalised fill value of each cell to fill
      const int nd = compact(XE_R, ND);
      for (int li = tid; li < nd; li += XNT) {
        const int r = LST[li] >> 8, c = LST[li] & 255;
        const int gx = x0 - 4 + c;
        float xv[9], xw[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int sc = min(max(gx + j - 4, T.wx0), T.wx1 - 1) - (x0 - 8);
          xv[j] = VV[r * XS_C + sc];
          xw[j] = VW[r * XS_C + sc];
        }
        const float2 s2 = gsum_ff2(gw, xv, xw);
        const float sv = s2.x, sw = s2.y;
        Sv[(r + 4) * XS_C + c + 4] = sw > 0.0f ? __fdiv_rn(sv, sw) : 0.0f;  // after every read of (d)
      }
      __syncthreads();
    }
    auto fe = [&](int gy, int gx) { return Sv[(gy - (y0 - 8)) * XS_C + (gx - (x0 - 8))]; };
    // (f) first derivatives around the unit (curvature) and (g) the outputs: both
    //     cell lists built in one pass, (g)'s after the derivative planes
    int* LOFF_G = reinterpret_cast<int*>(VV + XG_OFF);
    unsigned short* LST_G = reinterpret_cast<unsigned short*>(LOFF_G + XL_ROWS);
    // (g) lists the pixels recomputed; the other pixels keep the fast pass's values (no
    // NoData and no window edge in their stencil)
    auto out_rows = [&](int r) { return (AF[r + 4] >> 4) & ((1ull << FW) - 1ull); };
    int no;
    if (CURV) {
      // the derivatives within one cell of the pixels recomputed (D row r, column c = E row
      // r + 2, column c + 2); at the window edge the one-sided second differences of the
      // edge band reach two cells inward, through NoData too
      auto deriv_rows = [&](int r) {
        const unsigned long long a3 = AF[r + 1] | AF[r + 2] | AF[r + 3];
        unsigned long long m = (a3 >> 1) | (a3 >> 2) | (a3 >> 3);
        if (band) {
          const int gy = y0 - 2 + r;
          if (gy < T.wy0 + 4 || gy >= T.wy1 - 4) {
            m = ~0ull;
          } else {
            const int l1 = T.wx0 + 4 - (x0 - 2), h0 = T.wx1 - 4 - (x0 - 2);  // D columns [0, l1) and [h0, XD_C)
            if (l1 > 0) m |= l1 >= 64 ? ~0ull : ((1ull << l1) - 1ull);
            if (h0 < XD_C) m |= ~0ull << max(h0, 0);
          }
        }
        return m & ((1ull << XD_C) - 1ull);
      };
      // one warp scans each list; NV (free once the fills are done) keeps the derivative masks
      if (warp == 0) scan_rows(XD_R, deriv_rows, LOFF, NV);
      else if (warp == 1) scan_rows(SH, out_rows, LOFF_G, nullptr);
      __syncthreads();
      write_rows(XD_R, [&](int r) { return NV[r]; }, LOFF, LST);
      write_rows(SH, out_rows, LOFF_G, LST_G);
      __syncthreads();
      const int2 cnt = make_int2(LOFF[XL_ROWS - 1], LOFF_G[XL_ROWS - 1]);
      const int ndv = cnt.x;
      no = cnt.y;
      for (int li = tid; li < ndv; li += XNT) {
        const int r = LST[li] >> 8, c = LST[li] & 255, i = r * XD_C + c;
        const int gy = y0 - 2 + r, gx = x0 - 2 + c;
        float dx = qnan, dy = qnan;
        if (gy >= T.wy0 && gy < T.wy1 && gx >= T.wx0 && gx < T.wx1) {
          // correctly rounded: the second differences amplify their last bit (as in the fast pass)
          dx = deriv_d<true>(T.g1x, gx, T.wx0, T.wx1, [&](int k) { return fe(gy, gx + k); });
          dy = deriv_d<true>(T.g1y, gy, T.wy0, T.wy1, [&](int k) { return fe(gy + k, gx); });
        }
        DX[i] = dx;
        DY[i] = dy;
      }
      __syncthreads();
    } else {
      if (warp == 0) scan_rows(SH, out_rows, LOFF_G, nullptr);
      __syncthreads();
      write_rows(SH, out_rows, LOFF_G, LST_G);
      __syncthreads();
      no = LOFF_G[XL_ROWS - 1];
    }
    const Light L{A.lx, A.ly, A.lz, A.slope_unit};
    for (int li = tid; li < no; li += XNT) {
      const int r = LST_G[li] >> 8, c = LST_G[li] & 255;
      const int gy = y0 + r, gx = x0 + c;
      if (gy >= y1 || gx >= xo) continue;
      float o[FSG_STENCIL_NOUT];
      const float z0 = Sv[(r + 8) * XS_C + c + 8];
      if (z0 == z0) {
        float p, q, dxx = 0.f, dxy = 0.f, dyy = 0.f, dyx = 0.f;
        if (CURV) {
          auto dxa = [&](int yy, int xx) { return DX[(yy - (y0 - 2)) * XD_C + (xx - (x0 - 2))]; };
          auto dya = [&](int yy, int xx) { return DY[(yy - (y0 - 2)) * XD_C + (xx - (x0 - 2))]; };
          p = dxa(gy, gx);
          q = dya(gy, gx);
          dxx = deriv_d<true>(T.c2x, gx, T.wx0, T.wx1, [&](int k) { return dxa(gy, gx + k); });
          dxy = deriv_d<true>(T.c2y, gy, T.wy0, T.wy1, [&](int k) { return dxa(gy + k, gx); });
          dyy = deriv_d<true>(T.c2y, gy, T.wy0, T.wy1, [&](int k) { return dya(gy + k, gx); });
          if (OM & (1u << FSG_OUT_CURV_MEAN))
            dyx = deriv_d<true>(T.c2x, gx, T.wx0, T.wx1, [&](int k) { return dya(gy, gx + k); });
        } else {
          p = deriv_d<DIV>(T.g1x, gx, T.wx0, T.wx1, [&](int k) { return fe(gy, gx + k); });
          q = deriv_d<DIV>(T.g1y, gy, T.wy0, T.wy1, [&](int k) { return fe(gy + k, gx); });
        }
        float pz = p, qz = q;
        if ((OM & (1u << FSG_OUT_HILLSHADE)) && !A.z_is_one) {
          const float zf = A.z;
          pz = deriv_d<DIV>(T.g1x, gx, T.wx0, T.wx1, [&](int k) { return fmul(fe(gy, gx + k), zf); });
          qz = deriv_d<DIV>(T.g1y, gy, T.wy0, T.wy1, [&](int k) { return fmul(fe(gy + k, gx), zf); });
        }
        pixel_products(L, T.sx, T.sy, OM, p, q, pz, qz, dxx, dxy, dyy, dyx, o);
      } else {
#pragma unroll
        for (int kk = 0; kk < FSG_STENCIL_NOUT; ++kk) o[kk] = qnan;
      }
      char* optr[FSG_STENCIL_NOUT];
#pragma unroll
      for (int k = 0; k < FSG_STENCIL_NOUT; ++k) {
        if (!(OM & (1u << k))) continue;
        const PlaneK& P = A.planes[k];
        const int esz = ALLF32 ? 4 : (P.dtype == FSG_F32 ? 4 : (P.dtype == FSG_I16 ? 2 : 1));
        optr[k] = static_cast<char*>(P.ptr) + ((long long)(T.oy0 + gy - T.cy0) * P.ld + (T.ox0 + gx - T.cx0)) * esz;
      }
      store_pixel(A, OM, ALLF32, optr, o);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------- host
Axis make_axis(double step) {
  Axis a;
  a.d2 = (float)(2.0 * step);
  a.rcp = 1.0f / a.d2;  // host IEEE division: RN(1/d2)
  a.fa = (float)(-1.5 / step);
  a.fb = (float)(2.0 / step);
  a.fc = (float)(-0.5 / step);
  a.ba = (float)(0.5 / step);
  a.bb = (float)(-2.0 / step);
  a.bc = (float)(1.5 / step);
  return a;
}

// Step sizes of _nan_utils.py:67-72 (first derivatives) and
// _impl_curvature.py:263-268 (second derivatives).
void tile_steps(double pixel_size, double psx, double psy, double* g1x, double* g1y, double* c2x,
                double* c2y) {
  double fallback = pixel_size != 0.0 ? pixel_size : 1.0;
  double cx = psx, cy = psy;
  if (std::fabs(cy) < 1e-9) cy = fallback;
  if (std::fabs(cx) < 1e-9) cx = fallback;
  *c2x = cx;
  *c2y = cy;
  double gx = std::fabs(cx), gy = std::fabs(cy);
  if (gx < 1e-9) gx = fallback;
  if (gy < 1e-9) gy = fallback;
  *g1x = gx;
  *g1y = gy;
}

const double kGaussW[5] = {0x1.9884a307594fbp-2, 0x1.ef8eb9ad499bap-3, 0x1.ba4b99d1799abp-5,
                           0x1.22724cb7eb269p-8, 0x1.18a9c4fd536c6p-13};

}  // namespace

int validate_tiles(int32_t raster_h, int32_t raster_w, const fsg_tile* tiles, int32_t ntiles,
                   int min_window) {
  for (int t = 0; t < ntiles; ++t) {
    const fsg_tile& s = tiles[t];
    if (s.win_h < 0 || s.win_w < 0 || s.core_h < 0 || s.core_w < 0)
      return fail(FSG_ERR_INVALID, "tile %d: negative size", t);
    if (s.win_y0 < 0 || s.win_x0 < 0 || (int64_t)s.win_y0 + s.win_h > raster_h ||
        (int64_t)s.win_x0 + s.win_w > raster_w)
      return fail(FSG_ERR_INVALID, "tile %d: window outside the %d x %d raster", t, raster_h, raster_w);
    if (s.core_h == 0 || s.core_w == 0) continue;
    if (s.core_y0 < s.win_y0 || s.core_x0 < s.win_x0 || s.core_y0 + s.core_h > s.win_y0 + s.win_h ||
        s.core_x0 + s.core_w > s.win_x0 + s.win_w)
      return fail(FSG_ERR_INVALID, "tile %d: core outside its window", t);
    if (s.out_y0 < 0 || s.out_x0 < 0) return fail(FSG_ERR_INVALID, "tile %d: negative output origin", t);
    if (s.win_h < min_window || s.win_w < min_window)
      return fail(FSG_ERR_SHAPE,
                  "tile %d: window %d x %d too small to calculate a numerical gradient, at least "
                  "(edge_order + 1) = 3 elements are required",
                  t, s.win_h, s.win_w);
  }
  return FSG_OK;
}

}  // namespace fsg

namespace fsg {
// One fused-stencil job: every table and launch parameter, built on the host.
// The eager entry point uploads the tables into stream-ordered scratch and
// launches; a plan uploads them once into memory it owns, and each launch
// then only issues a memset and kernels (capturable in a CUDA graph).
constexpr size_t FAST_SMEM = sizeof(float) * (FSG_FAST_NT / 32) * RING * RW + 8 * (FSG_FAST_NT / 32) * RING;

// cuTensorMapEncodeTiled is a driver entry point: it is looked up through the runtime once, so
// the library loads (and its symbols resolve) where no driver is installed
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

struct StencilJob {
  bool empty = true, fast = false;
  StencilArgs A;
  std::vector<TileK> tk;
  void (*kern)(StencilArgs) = nullptr;
  int grid = 0;
  FastArgs F;
  std::vector<FastTile> ft;
  int units = 0, fgrid = 0, xgrid = 0;
  void (*fastk)(FastArgs) = nullptr;
  void (*fixk)(FastArgs) = nullptr;
  size_t tiles_bytes() const {
    return fast ? (sizeof(FastTile) * ft.size() + 255) & ~(size_t)255
                : (tk.size() > (size_t)INLINE_TILES ? (sizeof(TileK) * tk.size() + 255) & ~(size_t)255 : 0);
  }
  size_t device_bytes() const { return tiles_bytes() + (fast ? sizeof(unsigned) * ((size_t)NQ * units + 3) : 0); }
  // point the kernel arguments at the tables / fix-up list in `dev`
  void bind(void* dev) {
    if (fast) {
      unsigned* fix = reinterpret_cast<unsigned*>(static_cast<unsigned char*>(dev) + tiles_bytes());
      F.tiles = static_cast<const FastTile*>(dev);
      F.fix_count = fix;
      F.queue = fix + 1;
      F.fix_queue = fix + 2;
      F.fix_list = fix + 3;
    } else if (tk.size() > (size_t)INLINE_TILES) {
      A.tiles_dev = static_cast<const TileK*>(dev);
    }
  }
  // the host image of the tables (tiles_bytes() bytes at dst)
  void pack(char* dst) const {
    if (fast) std::memcpy(dst, ft.data(), sizeof(FastTile) * ft.size());
    else if (tk.size() > (size_t)INLINE_TILES) std::memcpy(dst, tk.data(), sizeof(TileK) * tk.size());
  }
  int upload(void* dev, cudaStream_t s) const {
    if (fast) FSG_UPLOAD(dev, ft.data(), sizeof(FastTile) * ft.size(), s);
    else if (tk.size() > (size_t)INLINE_TILES)
      FSG_UPLOAD(dev, tk.data(), sizeof(TileK) * tk.size(), s);
    return FSG_OK;
  }
  // the streaming pass's tensor map of the raster (once its device pointer is final): a 2-D
  // float32 map with RBOX x 1 boxes; without a 16-byte aligned base and row pitch the pass
  // fills its ring with cp.async instead
  void encode_tmap() {
    F.use_tma = 0;
    if (!fast || !F.raster || A.rw < 1 || A.rh < 1) return;
    if (((uintptr_t)F.raster & 15) != 0 || (F.ld & 3) != 0) return;
    const char* off = getenv("FSG_NO_TMA");
    if (off && off[0] == '1') return;
    cuuint64_t dims[2] = {(cuuint64_t)A.rw, (cuuint64_t)A.rh};
    cuuint64_t strides[1] = {(cuuint64_t)F.ld * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)RBOX, 1};
    cuuint32_t estr[2] = {1, 1};
    const EncodeTiledFn enc = encode_tiled_fn();
    if (!enc) return;
    const CUresult r = enc(&F.tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(F.raster), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    F.use_tma = r == CUDA_SUCCESS ? 1 : 0;
  }
  // launches only (no host memory involved)
  int enqueue(cudaStream_t s) const {
    if (empty) return FSG_OK;
    if (fast) {
      FSG_CUDA(cudaMemsetAsync(F.fix_count, 0, 3 * sizeof(unsigned), s));  // fix-up count and both queue heads
      timing_mark(s, true);
      fastk<<<fgrid, FSG_FAST_NT, FAST_SMEM, s>>>(F);
      timing_mark(s, false);
      FSG_LAUNCHED(1);
      fixk<<<xgrid, XNT, FIX_SMEM, s>>>(F);
      FSG_LAUNCHED(1);
      return FSG_OK;
    }
    kern<<<grid, NT, SMEM_BYTES, s>>>(A);
    FSG_LAUNCHED(1);
    return FSG_OK;
  }
};

static int stencil_prepare(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                           const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                           const fsg_plane* planes, StencilJob& J) {
  if (!params || !planes || (ntiles > 0 && !tiles)) return fail(FSG_ERR_INVALID, "null argument");
  if (ntiles < 0 || raster_h < 0 || raster_w < 0) return fail(FSG_ERR_INVALID, "negative size");
  if (ld < raster_w) return fail(FSG_ERR_INVALID, "row pitch %lld < width %d", (long long)ld, raster_w);
  if (params->slope_unit < 0 || params->slope_unit > 2)
    return fail(FSG_ERR_INVALID, "slope_unit %d", params->slope_unit);
  unsigned outmask = 0;
  for (int o = 0; o < FSG_STENCIL_NOUT; ++o) {
    if (!planes[o].ptr) continue;
    if (planes[o].dtype < FSG_F32 || planes[o].dtype > FSG_I16)
      return fail(FSG_ERR_DTYPE, "plane %d: dtype %d", o, planes[o].dtype);
    if (planes[o].dtype != FSG_F32) {  // codes are clamped to [q_min, q_max]: they must fit the type
      const int lo = planes[o].dtype == FSG_U8 ? 0 : -32768, hi = planes[o].dtype == FSG_U8 ? 255 : 32767;
      if (planes[o].q_min < lo || planes[o].q_max > hi)
        return fail(FSG_ERR_INVALID, "plane %d: code range [%d, %d] outside [%d, %d]", o, planes[o].q_min,
                    planes[o].q_max, lo, hi);
    }
    outmask |= 1u << o;
  }
  if (!outmask) return fail(FSG_ERR_INVALID, "no output plane requested");
  int st = validate_tiles(raster_h, raster_w, tiles, ntiles, 3);
  if (st) return st;

  StencilArgs& A = J.A;
  std::memset(&A, 0, sizeof(A));
  A.raster = raster_dev;
  A.ld = ld;
  A.rh = raster_h;
  A.rw = raster_w;
  double alt = params->altitude * M_PI / 180.0;
  double az = params->azimuth * M_PI / 180.0;
  A.lx = (float)(std::sin(az) * std::cos(alt));
  A.ly = (float)(std::cos(az) * std::cos(alt));
  A.lz = (float)std::sin(alt);
  A.z = (float)params->z_factor;
  A.z_is_one = params->z_factor == 1.0;
  A.ndf = (float)params->nodata;
  A.has_nodata = params->has_nodata != 0;
  A.slope_unit = params->slope_unit;
  A.outmask = outmask;
  for (int j = 0; j < 5; ++j) {
    A.gw_hi[j] = (float)kGaussW[j];
    A.gw_lo[j] = (float)(kGaussW[j] - (double)A.gw_hi[j]);
  }
  for (int o = 0; o < FSG_STENCIL_NOUT; ++o) {
    A.planes[o].ptr = planes[o].ptr;
    A.planes[o].ld = planes[o].ld;
    A.planes[o].dtype = planes[o].dtype;
    A.planes[o].qa = planes[o].q_a;
    A.planes[o].qb = planes[o].q_b;
    A.planes[o].qmin = planes[o].q_min;
    A.planes[o].qmax = planes[o].q_max;
  }
  std::vector<TileK>& tk = J.tk;
  tk.clear();
  tk.reserve(ntiles);
  int total = 0;
  for (int t = 0; t < ntiles; ++t) {
    const fsg_tile& s = tiles[t];
    if (s.core_h == 0 || s.core_w == 0) continue;
    TileK k;
    k.wy0 = s.win_y0;
    k.wx0 = s.win_x0;
    k.wy1 = s.win_y0 + s.win_h;
    k.wx1 = s.win_x0 + s.win_w;
    k.cy0 = s.core_y0;
    k.cx0 = s.core_x0;
    k.cy1 = s.core_y0 + s.core_h;
    k.cx1 = s.core_x0 + s.core_w;
    k.oy0 = s.out_y0;
    k.ox0 = s.out_x0;
    k.nbx = (s.core_w + TX - 1) / TX;
    int nby = (s.core_h + TY - 1) / TY;
    k.block0 = total;
    total += k.nbx * nby;
    double g1x, g1y, c2x, c2y;
    tile_steps(params->pixel_size, s.pixel_scale_x, s.pixel_scale_y, &g1x, &g1y, &c2x, &c2y);
    k.g1x = make_axis(g1x);
    k.g1y = make_axis(g1y);
    k.c2x = make_axis(c2x);
    k.c2y = make_axis(c2y);
    k.sign_x = s.pixel_scale_x >= 0.0 ? 1.0f : -1.0f;
    k.sign_y = s.pixel_scale_y >= 0.0 ? 1.0f : -1.0f;
    tk.push_back(k);
  }
  J.empty = total == 0;
  if (J.empty) return FSG_OK;
  A.ntiles = (int)tk.size();
  A.total_blocks = total;
  if (A.ntiles <= INLINE_TILES) std::copy(tk.begin(), tk.end(), A.inl);
  DeviceInfo di;
  st = device_info(&di);
  if (st) return st;
  const bool curv = (outmask & ((1u << FSG_OUT_CURV_MEAN) | (1u << FSG_OUT_CURV_GAUSSIAN) |
                                (1u << FSG_OUT_CURV_PLANFORM) | (1u << FSG_OUT_CURV_PROFILE))) != 0;
  J.kern = curv ? stencil_kernel<true, 0u> : stencil_kernel<false, 0u>;
  void (*fast)(FastArgs) = nullptr;
  void (*fixup)(FastArgs) = nullptr;
  constexpr unsigned HS = 1u << FSG_OUT_HILLSHADE, SL = 1u << FSG_OUT_SLOPE, CM = 1u << FSG_OUT_CURV_MEAN,
                     CG = 1u << FSG_OUT_CURV_GAUSSIAN, CP = 1u << FSG_OUT_CURV_PLANFORM,
                     CR = 1u << FSG_OUT_CURV_PROFILE, DXY = (1u << FSG_OUT_DX) | (1u << FSG_OUT_DY);
  bool allf32 = true, allu8 = true;
  for (int o = 0; o < FSG_STENCIL_NOUT; ++o)
    if ((outmask >> o) & 1u) {
      allf32 = allf32 && planes[o].dtype == FSG_F32;
      allu8 = allu8 && planes[o].dtype == FSG_U8;
    }
  switch (outmask) {
#define FSG_CASE(M, C)                                                                         \
  case (M):                                                                                    \
    if (((M) & HS) && A.z_is_one)                                                              \
      fast = allf32 ? stencil_fast_kernel<C, (M), 1, true>                                     \
                    : (allu8 ? stencil_fast_kernel<C, (M), 2, true> : stencil_fast_kernel<C, (M), 0, true>); \
    else                                                                                       \
      fast = allf32 ? stencil_fast_kernel<C, (M), 1, false> : stencil_fast_kernel<C, (M), 0, false>; \
    fixup = allf32 ? stencil_fixup_kernel<(M), true> : stencil_fixup_kernel<(M), false>;       \
    break;
    FSG_CASE(HS | SL | CP | CR, true)
    FSG_CASE(HS | SL | CM | CG | CP | CR, true)
    FSG_CASE(HS, false)
    FSG_CASE(SL, false)
    FSG_CASE(HS | SL, false)
    FSG_CASE(CM, true)
    FSG_CASE(CG, true)
    FSG_CASE(CP, true)
    FSG_CASE(CR, true)
    FSG_CASE(DXY, false)
#undef FSG_CASE
    default: break;
  }
  J.fast = fast != nullptr;
  if (J.fast) {
    // fast streaming pass over every tile, then the exact fix-up of the quarters it flagged
    J.ft.clear();
    int units = 0;
    for (const TileK& k : tk) {
      FastTile f;
      f.wy0 = k.wy0; f.wx0 = k.wx0; f.wy1 = k.wy1; f.wx1 = k.wx1;
      f.cy0 = k.cy0; f.cx0 = k.cx0; f.cy1 = k.cy1; f.cx1 = k.cx1;
      f.oy0 = k.oy0; f.ox0 = k.ox0;
      const int cw = k.cx1 - k.cx0, ch = k.cy1 - k.cy0;
      f.nstrip = std::max(1, (cw + SW - 1) / SW);
      f.unit0 = units;
      units += f.nstrip * ((ch + SH - 1) / SH);
      f.g1x = k.g1x; f.g1y = k.g1y; f.c2x = k.c2x; f.c2y = k.c2y;
      f.sx = k.sign_x; f.sy = k.sign_y;
      J.ft.push_back(f);
    }
    if ((unsigned)units > FIX_UNIT) return fail(FSG_ERR_UNSUPPORTED, "%d stencil units exceed the fix-up list's index range", units);
    FastArgs& F = J.F;
    std::memset(&F, 0, sizeof(F));
    F.raster = A.raster;
    F.ld = A.ld;
    F.lx = A.lx; F.ly = A.ly; F.lz = A.lz; F.z = A.z;
    F.z_is_one = A.z_is_one;
    F.ndf = A.ndf;
    F.has_nodata = A.has_nodata;
    F.slope_unit = A.slope_unit;
    F.ntiles = (int)J.ft.size();
    F.total_units = units;
    for (int j = 0; j < 5; ++j) F.gw[j] = {A.gw_hi[j], A.gw_lo[j]};
    std::copy(A.planes, A.planes + FSG_STENCIL_NOUT, F.planes);
    for (int o = 0; o < FSG_STENCIL_NOUT; ++o) {
      F.qlim[o][0] = (float)A.planes[o].qmin;
      F.qlim[o][1] = (float)A.planes[o].qmax;
    }
    J.units = units;
    J.fastk = fast;
    J.fixk = fixup;
    int fper = 0;
    FSG_CUDA(cudaFuncSetAttribute(fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FAST_SMEM));
    FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fper, fast, FSG_FAST_NT, FAST_SMEM));
    J.fgrid = std::min((units + FSG_FAST_NT / 32 - 1) / (FSG_FAST_NT / 32), di.sms * std::max(1, fper));  // one unit per warp
    FSG_CUDA(cudaFuncSetAttribute(fixup, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FIX_SMEM));
    int xper = 0;
    FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&xper, fixup, XNT, FIX_SMEM));
    J.xgrid = std::min(NQ * units, di.sms * std::max(1, xper));
    return FSG_OK;
  }
  FSG_CUDA(cudaFuncSetAttribute(J.kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
  FSG_CUDA(cudaFuncSetAttribute(J.kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int per_sm = 0;
  FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, J.kern, NT, SMEM_BYTES));
  if (per_sm < 1) per_sm = 1;
  J.grid = std::min(total, di.sms * per_sm);
  return FSG_OK;
}

// A prepared fused-stencil launch over fixed buffers and tiles.
struct StencilPlan final : fsg_plan {
  StencilJob J;
  void* dev = nullptr;
  ~StencilPlan() override {
    if (dev) cudaFree(dev);
  }
  int launch(cudaStream_t s) override { return J.enqueue(s); }
};
}  // namespace fsg

extern "C" int fsg_stencil(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                           const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                           const fsg_plane* planes, void* stream) {
  using namespace fsg;
  StencilJob J;
  int st = stencil_prepare(raster_dev, ld, raster_h, raster_w, tiles, ntiles, params, planes, J);
  if (st || J.empty) return st;
  J.encode_tmap();
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch scratch;
  const size_t bytes = J.device_bytes();
  if (bytes) {
    st = scratch.alloc(bytes, s);
    if (st) return st;
    J.bind(scratch.ptr);
    st = J.upload(scratch.ptr, s);
    if (st) return st;
  }
  return J.enqueue(s);
}

extern "C" int fsg_stencil_plan(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                                const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                                const fsg_plane* planes, fsg_plan** plan) {
  using namespace fsg;
  if (!plan) return fail(FSG_ERR_INVALID, "null plan pointer");
  *plan = nullptr;
  StencilPlan* P = new StencilPlan();
  int st = stencil_prepare(raster_dev, ld, raster_h, raster_w, tiles, ntiles, params, planes, P->J);
  if (!st) P->J.encode_tmap();
  const size_t bytes = st ? 0 : P->J.device_bytes();
  if (!st && bytes) {
    cudaError_t e = cudaMalloc(&P->dev, bytes);
    if (e != cudaSuccess) {
      P->dev = nullptr;
      st = cuda_fail(e, "cudaMalloc(plan)");
    } else {
      P->J.bind(P->dev);
      st = P->J.upload(P->dev, nullptr);
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

// ------------------------------------------------------ host-buffer loop
// Host-buffer tile loop of the fused stencil: the single-device equivalent of
// process_dem_tiles' per-tile read -> H2D -> compute -> D2H cycle
// (core/tile_processor.py:822-1024, :1629-1683), with the three stages of
// consecutive batches overlapped.
//
// Consecutive tiles that form one row band of the grid (same core rows, cores
// side by side, one output offset) are one batch: the union of their windows
// goes down in one copy (one contiguous block when the band spans the
// raster's full width), one prepared stencil job covers all of its tiles, and
// each plane's band of cores comes back in one copy.  Other tiles are batches
// of one.  All jobs are prepared, and their tile tables uploaded in one copy,
// before the loop, which then issues only pinned copies and launches.
// Batches are assigned round-robin to NSLOT slots; each slot owns a
// device window buffer, one device buffer per requested plane and a stream,
// so the H2D copy of one batch, the kernels of the previous one and the D2H
// copies of the one before that run concurrently (separate copy engines for
// the two directions).  The slots' streams are ordered after, and joined back
// into, the caller's stream with events.
namespace fsg {
namespace {

constexpr int NSLOT = 3;
constexpr size_t kBandSlotBytes = (size_t)6 << 30;  // larger bands run tile by tile

struct SlotStreams {
  cudaStream_t s[NSLOT] = {};
  cudaEvent_t done[NSLOT] = {};
  cudaEvent_t start = nullptr;
};
std::mutex g_slot_mutex;
SlotStreams g_slots[64];
bool g_slots_ready[64] = {};

int slot_streams(SlotStreams** out) {
  int dev = 0;
  FSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FSG_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_slot_mutex);
  if (!g_slots_ready[dev]) {
    SlotStreams& S = g_slots[dev];
    for (int i = 0; i < NSLOT; ++i) {
      FSG_CUDA(cudaStreamCreateWithFlags(&S.s[i], cudaStreamNonBlocking));
      FSG_CUDA(cudaEventCreateWithFlags(&S.done[i], cudaEventDisableTiming));
    }
    FSG_CUDA(cudaEventCreateWithFlags(&S.start, cudaEventDisableTiming));
    g_slots_ready[dev] = true;
  }
  *out = &g_slots[dev];
  return FSG_OK;
}

size_t esize(int dtype) { return dtype == FSG_F32 ? 4 : (dtype == FSG_I16 ? 2 : 1); }

// A batch: tiles [t0, t1) with the union of their windows and of their cores.
struct Batch {
  int t0, t1;
  int wy0, wx0, wh, ww;  // window union (raster coords)
  int cy0, cx0, ch, cw;  // core union (raster coords)
  int oy0, ox0;          // output coords of (cy0, cx0)
};

std::vector<Batch> make_batches(const fsg_tile* tiles, int ntiles, int nplanes_f32_equiv) {
  std::vector<Batch> out;
  int t = 0;
  while (t < ntiles) {
    const fsg_tile& A = tiles[t];
    Batch b{t, t + 1, A.win_y0, A.win_x0, A.win_h, A.win_w, A.core_y0, A.core_x0, A.core_h, A.core_w, A.out_y0,
            A.out_x0};
    int u = t + 1;
    while (u < ntiles) {
      const fsg_tile& B = tiles[u];
      const fsg_tile& P = tiles[u - 1];
      // same core rows, next core directly to the right, same output offset
      if (B.core_y0 != A.core_y0 || B.core_h != A.core_h || B.core_x0 != P.core_x0 + P.core_w ||
          B.out_y0 - B.core_y0 != A.out_y0 - A.core_y0 || B.out_x0 - B.core_x0 != A.out_x0 - A.core_x0 ||
          B.core_w == 0)
        break;
      const int wy1 = std::max(b.wy0 + b.wh, B.win_y0 + B.win_h), wx1 = std::max(b.wx0 + b.ww, B.win_x0 + B.win_w);
      const int wy0 = std::min(b.wy0, B.win_y0), wx0 = std::min(b.wx0, B.win_x0);
      const size_t bytes = (size_t)(wy1 - wy0) * (wx1 - wx0) * 4 +
                           (size_t)b.ch * (b.cw + B.core_w) * 4 * (size_t)nplanes_f32_equiv;
      if (bytes > kBandSlotBytes) break;
      b.wy0 = wy0;
      b.wx0 = wx0;
      b.wh = wy1 - wy0;
      b.ww = wx1 - wx0;
      b.cw += B.core_w;
      b.t1 = ++u;
    }
    out.push_back(b);
    t = u;
  }
  return out;
}

}  // namespace
}  // namespace fsg


extern "C" int fsg_stencil_host(const float* raster_host, int64_t ld, int32_t raster_h, int32_t raster_w,
                                const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                                const fsg_plane* planes_host, void* stream) {
  using namespace fsg;
  if (!raster_host || !params || !planes_host || (ntiles > 0 && !tiles)) return fail(FSG_ERR_INVALID, "null argument");
  if (ntiles < 0 || raster_h < 0 || raster_w < 0 || ld < raster_w) return fail(FSG_ERR_INVALID, "bad raster shape");
  int st = validate_tiles(raster_h, raster_w, tiles, ntiles, 3);
  if (st) return st;
  std::vector<int> req;
  for (int o = 0; o < FSG_STENCIL_NOUT; ++o)
    if (planes_host[o].ptr) {
      if (planes_host[o].dtype < FSG_F32 || planes_host[o].dtype > FSG_I16)
        return fail(FSG_ERR_DTYPE, "plane %d: dtype %d", o, planes_host[o].dtype);
      req.push_back(o);
    }
  if (req.empty()) return fail(FSG_ERR_INVALID, "no output plane requested");
  if (ntiles == 0) return FSG_OK;
  const std::vector<Batch> batches = make_batches(tiles, ntiles, (int)req.size());
  int maxwh = 0, maxww = 0, maxch = 0, maxcw = 0;
  for (const Batch& b : batches) {
    maxwh = std::max(maxwh, b.wh);
    maxww = std::max(maxww, b.ww);
    maxch = std::max(maxch, b.ch);
    maxcw = std::max(maxcw, b.cw);
  }
  if (maxch == 0 || maxcw == 0) return FSG_OK;
  const int64_t wpitch = ((int64_t)maxww + 31) & ~(int64_t)31;  // elements, 128-byte rows
  const int64_t cpitch = ((int64_t)maxcw + 127) & ~(int64_t)127;  // elements of each core plane row
  size_t slot_bytes = (size_t)wpitch * maxwh * sizeof(float);
  for (int o : req) slot_bytes += (size_t)cpitch * maxch * esize(planes_host[o].dtype) + 256;
  slot_bytes = (slot_bytes + 255) & ~(size_t)255;
  cudaStream_t caller = (cudaStream_t)stream;
  SlotStreams* S = nullptr;
  st = slot_streams(&S);
  if (st) return st;
  const int nslot = std::min<int>(NSLOT, (int)batches.size());
  // every batch prepared first (its window and planes are its slot's buffers), the tile tables
  // of all batches uploaded in one copy: inside the loop only pinned copies and launches remain
  // (a pageable host-to-device copy synchronises its stream, which would stall the pipeline)
  std::vector<StencilJob> jobs(batches.size());
  std::vector<size_t> job_off(batches.size(), 0);
  std::vector<int64_t> bpitch(batches.size(), 0);
  std::vector<std::array<int64_t, FSG_STENCIL_NOUT>> opitch(batches.size());
  std::vector<std::array<char*, FSG_STENCIL_NOUT>> optr(batches.size());
  size_t tables = 0;
  std::vector<fsg_tile> local;
  const size_t slots_total = slot_bytes * nslot;
  // pass 1: layout (device pointers are bound after the allocation)
  for (size_t bi = 0; bi < batches.size(); ++bi) {
    const Batch& B = batches[bi];
    if (B.ch == 0 || B.cw == 0) continue;
    bpitch[bi] = (B.wx0 == 0 && B.ww == raster_w && ld == raster_w) ? (int64_t)raster_w : wpitch;
    for (int o : req) opitch[bi][o] = (B.cw == planes_host[o].ld) ? (int64_t)B.cw : cpitch;
  }
  StreamScratch scratch;
  // the job tables' sizes depend on the tiles only: prepare against placeholder pointers, then rebind
  for (size_t bi = 0; bi < batches.size(); ++bi) {
    const Batch& B = batches[bi];
    if (B.ch == 0 || B.cw == 0) continue;
    const int k = (int)(bi % nslot);
    fsg_plane dev_planes[FSG_STENCIL_NOUT];
    std::memset(dev_planes, 0, sizeof(dev_planes));
    size_t p = (size_t)wpitch * maxwh * sizeof(float);
    for (int o : req) {
      dev_planes[o] = planes_host[o];
      dev_planes[o].ptr = reinterpret_cast<void*>((uintptr_t)(slot_bytes * k + p + 1));  // offset + 1 (non-null)
      dev_planes[o].ld = opitch[bi][o];
      p += ((size_t)cpitch * maxch * esize(planes_host[o].dtype) + 255) & ~(size_t)255;
    }
    local.assign(tiles + B.t0, tiles + B.t1);
    for (fsg_tile& T : local) {
      T.win_y0 -= B.wy0;
      T.win_x0 -= B.wx0;
      T.core_y0 -= B.wy0;
      T.core_x0 -= B.wx0;
      T.out_y0 = (T.core_y0 + B.wy0) - B.cy0;
      T.out_x0 = (T.core_x0 + B.wx0) - B.cx0;
    }
    const float* win_off = reinterpret_cast<const float*>((uintptr_t)(slot_bytes * k + 1));
    st = stencil_prepare(win_off, bpitch[bi], B.wh, B.ww, local.data(), (int)local.size(), params, dev_planes,
                         jobs[bi]);
    if (st) return st;
    job_off[bi] = slots_total + tables;
    tables += (jobs[bi].device_bytes() + 255) & ~(size_t)255;
  }
  st = scratch.alloc(slots_total + tables, caller);
  if (st) return st;
  char* base = static_cast<char*>(scratch.ptr);
  std::vector<char> image(std::max<size_t>(tables, 1));
  auto rebase = [&](const void* off) { return base + ((uintptr_t)off - 1); };
  for (size_t bi = 0; bi < batches.size(); ++bi) {
    const Batch& B = batches[bi];
    if (B.ch == 0 || B.cw == 0) continue;
    StencilJob& J = jobs[bi];
    for (int o : req) {
      optr[bi][o] = rebase(J.A.planes[o].ptr);
      J.A.planes[o].ptr = optr[bi][o];
      J.F.planes[o].ptr = optr[bi][o];
    }
    J.A.raster = reinterpret_cast<const float*>(rebase(J.A.raster));
    J.F.raster = J.A.raster;
    J.encode_tmap();
    J.bind(base + job_off[bi]);
    J.pack(image.data() + (job_off[bi] - slots_total));
  }
  if (tables) FSG_UPLOAD(base + slots_total, image.data(), tables, caller);
  FSG_CUDA(cudaEventRecord(S->start, caller));
  for (int i = 0; i < nslot; ++i) FSG_CUDA(cudaStreamWaitEvent(S->s[i], S->start, 0));
  int status = FSG_OK;
  for (size_t bi = 0; bi < batches.size() && status == FSG_OK; ++bi) {
    const Batch& B = batches[bi];
    if (B.ch == 0 || B.cw == 0) continue;
    const int k = (int)(bi % nslot);
    cudaStream_t s = S->s[k];
    float* win = reinterpret_cast<float*>(base + slot_bytes * k);
    // H2D: the window union (one contiguous block for a full-width band)
    cudaError_t e = cudaMemcpy2DAsync(win, bpitch[bi] * sizeof(float), raster_host + (int64_t)B.wy0 * ld + B.wx0,
                                      ld * sizeof(float), (size_t)B.ww * sizeof(float), B.wh,
                                      cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      status = cuda_fail(e, "cudaMemcpy2DAsync(H2D window)");
      break;
    }
    status = jobs[bi].enqueue(s);
    if (status) break;
    // D2H: the band of cores of every plane, into the caller's planes at (oy0, ox0)
    for (int o : req) {
      const size_t es = esize(planes_host[o].dtype);
      char* dst = static_cast<char*>(planes_host[o].ptr) + ((int64_t)B.oy0 * planes_host[o].ld + B.ox0) * es;
      e = cudaMemcpy2DAsync(dst, planes_host[o].ld * es, optr[bi][o], opitch[bi][o] * es, (size_t)B.cw * es, B.ch,
                            cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) {
        status = cuda_fail(e, "cudaMemcpy2DAsync(D2H plane)");
        break;
      }
    }
  }
  for (int i = 0; i < nslot; ++i) {
    cudaEventRecord(S->done[i], S->s[i]);
    cudaStreamWaitEvent(caller, S->done[i], 0);
  }
  return status;
}

extern "C" int fsg_kernel_errors(uint32_t* flags) {
  using namespace fsg;
  if (!flags) return fail(FSG_ERR_INVALID, "null argument");
  unsigned v = 0;
  FSG_CUDA(cudaMemcpyFromSymbol(&v, g_kernel_errors, sizeof(v)));
  const unsigned zero = 0;
  FSG_CUDA(cudaMemcpyToSymbol(g_kernel_errors, &zero, sizeof(zero)));
  unsigned t = 0;
  const int st = tc_take_errors(&t);
  if (st) return st;
  *flags = v | t;
  return FSG_OK;
}
