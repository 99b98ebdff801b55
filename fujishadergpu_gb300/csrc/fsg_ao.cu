// Ambient occlusion: the reference's stylised screen-space occlusion estimate.
//
// Reference semantics (algorithms/_impl_ambient_occlusion.py:32-121), per tile
// window (the reference's block):
//   sample rings r = radius * (0.25, 0.5, 0.75, 1.0), ring after ring; per ring the
//   num_samples directions theta_i = 2*pi*i/n (np.linspace endpoint=False) with
//   offsets (np.round(r cos), np.round(r sin)) (half to even), (0, 0) skipped;
//   the block is edge-padded (:70, :88), so a sample beyond the window takes the
//   window's nearest border value;
//   occlusion = min(max(atan((z_s - z) / d), 0) / (pi/4), 1) * (1 - 0.3 * ring)
//   with d = max(hypot(dx |sx|, dy |sy|), 1e-9) (:90-100), summed where z_s and z
//   are both valid, divided by max(count, 1) (:102-107);
//   ao = clip(1 - mean * intensity, 0, 1), 1 at NoData cells, Gaussian sigma 1
//   ('nearest' at the window edges; scipy's separable float64 correlate, axis 0
//   then axis 1 with a float32 intermediate) (:109-116); ao^(1/2.2); NaN at NoData
//   cells (:118-119); the optional display stretch max((v - p1) / (p99 - p1), 0)
//   (algorithms/tile/dask_bridge.py:173-203); the output encoding.
//
// Two kernels per call:
//   ao_field_kernel  the AO values before the Gaussian over each tile's field
//                    region (the core widened by the filter's 4-pixel reach,
//                    clipped to the window) into scratch.  A CTA stages its
//                    64 x 32 pixel block plus the sample reach in shared memory
//                    with coordinates clamped to the window (the edge padding),
//                    so every sample is one unconditional shared-memory load;
//                    a thread evaluates two columns (x, x + 32) of four rows with
//                    paired FP32 arithmetic.  Blocks without NoData skip the
//                    validity bookkeeping (count = number of samples).
//   ao_finish_kernel the separable Gaussian (compensated float32 dot products)
//                    from a shared-memory tile of the field, gamma, NaN,
//                    stretch and the store.
// Reaches too large for shared memory read the raster directly (clamped loads).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fsg_common.cuh"

namespace fsg {
namespace {

constexpr int AX = 32, AY = 8, ARPT = 4;      // threads 32 x 8; a thread: 4 rows x 2 columns
constexpr int APW = 2 * AX, APH = AY * ARPT;  // pixels per block: 64 x 32
constexpr int GR = 4;                         // Gaussian sigma 1 radius (int(4 sigma + 0.5))
constexpr int FTW = APW + 2 * GR, FTH = APH + 2 * GR;  // finish tile: 72 x 40

struct AoSample {
  short ox, oy;
  float r;   // RN(1 / f32(d))
  float df;  // f32(1 - 0.3 * ring)
};

struct FieldReg {
  int y0, x0, h, w;  // raster coords of a tile's field region
};

struct AoArgs {
  const float* raster;
  long long ld;
  float ndf;
  int has_nodata;
  int ns;                    // samples per tile
  int reach;                 // max(|ox|, |oy|) over the samples
  int spitch;                // staged row pitch (floats); 0 = direct raster loads
  float intensity;
  const AoSample* samples;   // [ntiles * ns]: per tile its own distance table
  const fsg_tile* tiles;
  const FieldReg* freg;      // per tile: field region
  const long long* foff;     // per tile: first element of its field in `field`
  const int* fblock0;        // per tile: first field block
  const int* oblock0;        // per tile: first output block
  int ntiles, field_blocks, out_blocks;
  float* field;
  FF gw[GR + 1];             // Gaussian weights, centre first
  float lo, scale;           // display stretch (scale <= 0: none)
  void* out;
  long long old;
  int odtype;
  float qa, qb;
  int qmin, qmax;
};

__device__ __forceinline__ int tile_of(const int* first, int n, int blk) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= blk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ float load_clamped(const AoArgs& A, const fsg_tile& T, int y, int x) {
  y = min(max(y, T.win_y0), T.win_y0 + T.win_h - 1);
  x = min(max(x, T.win_x0), T.win_x0 + T.win_w - 1);
  const float v = __ldg(A.raster + (long long)y * A.ld + x);
  return is_nodata(v, A.ndf, A.has_nodata != 0) ? __int_as_float(0x7fc00000) : v;
}

typedef float2 f2;
__device__ __forceinline__ f2 S2(float a) { return make_float2(a, a); }

// One sample for the pixel pair: the elevation ratio (z_s - z) / d clamped to
// [0, 1], and the normalised occlusion min(atan(t) / (pi/4), 1) as t P(t^2),
// P of degree 6 fitted to atan(t)/t on [0, 1] (Lawson's iteratively reweighted
// least squares on Chebyshev nodes; |error| 2.5e-7 rad) with its coefficients
// scaled by 4/pi (1 - 2^-21): the scale keeps the value at t = 1 at most 1 (the
// reference's cap); evaluated in float32 the normalised occlusion is within
// 9e-7 of the exact one, far inside the 1e-5 output tolerance.  The saturating
// multiply also maps NaN (a NoData sample) to 0, so an invalid sample adds
// nothing.
constexpr double OCC_K = 1.27323954473516268615 * (1.0 - 1.0 / 2097152.0);
__device__ __forceinline__ f2 occlusion2(f2 v, f2 nz, float r) {
  const f2 d = __fadd2_rn(v, nz);
  const f2 t = make_float2(__saturatef(__fmul_rn(d.x, r)), __saturatef(__fmul_rn(d.y, r)));
  const f2 t2 = __fmul2_rn(t, t);
  f2 p = S2((float)(0x1.be6aeb6befd0ep-8 * OCC_K));
  p = __ffma2_rn(t2, p, S2((float)(-0x1.134927f17b444p-5 * OCC_K)));
  p = __ffma2_rn(t2, p, S2((float)(0x1.4623789788144p-4 * OCC_K)));
  p = __ffma2_rn(t2, p, S2((float)(-0x1.0f04d31a45d7cp-3 * OCC_K)));
  p = __ffma2_rn(t2, p, S2((float)(0x1.95aa000bc32efp-3 * OCC_K)));
  p = __ffma2_rn(t2, p, S2((float)(-0x1.552b7b387fd09p-2 * OCC_K)));
  p = __ffma2_rn(t2, p, S2((float)(0x1.ffff7d868299ep-1 * OCC_K)));
  return __fmul2_rn(t, p);
}

template <bool STAGED>
__global__ void __launch_bounds__(AX * AY) ao_field_kernel(const __grid_constant__ AoArgs A) {
  extern __shared__ __align__(16) unsigned char ao_smem[];
  AoSample* ss = reinterpret_cast<AoSample*>(ao_smem);
  int* soff = reinterpret_cast<int*>(ss + A.ns);
  float* zs = reinterpret_cast<float*>(soff + ((A.ns + 3) & ~3));
  const int tid = threadIdx.y * AX + threadIdx.x;
  const int R = A.reach;
  int loaded = -1;
  for (int blk = blockIdx.x; blk < A.field_blocks; blk += gridDim.x) {
    const int t = tile_of(A.fblock0, A.ntiles, blk);
    const fsg_tile T = A.tiles[t];
    const FieldReg E = A.freg[t];
    const int nbx = (E.w + APW - 1) / APW;
    const int lb = blk - A.fblock0[t];
    const int by = lb / nbx, bx = lb - by * nbx;
    const int bx0 = E.x0 + bx * APW, by0 = E.y0 + by * APH;
    __syncthreads();  // the previous block's readers are done with the tables
    if (t != loaded) {
      const AoSample* S = A.samples + (size_t)t * A.ns;
      for (int i = tid; i < A.ns; i += AX * AY) {
        const AoSample s = S[i];
        ss[i] = s;
        soff[i] = STAGED ? (int)s.oy * A.spitch + (int)s.ox : 0;
      }
      loaded = t;
    }
    bool nan_seen = false;
    if (STAGED) {
      const int sw = APW + 2 * R, sh = APH + 2 * R;
      for (int i = tid; i < sw * sh; i += AX * AY) {
        const int r = i / sw, c = i - (i / sw) * sw;
        const float v = load_clamped(A, T, by0 - R + r, bx0 - R + c);
        nan_seen |= v != v;
        zs[r * A.spitch + c] = v;
      }
    }
    const bool any_nan = STAGED ? __syncthreads_or(nan_seen) != 0 : true;
    if (!STAGED) __syncthreads();
    const int yb = by0 + threadIdx.y * ARPT;
    const int xa = bx0 + threadIdx.x, xb = xa + AX;
    f2 nz[ARPT], tot[ARPT], cnt[ARPT];
    int ci[ARPT];
#pragma unroll
    for (int k = 0; k < ARPT; ++k) {
      ci[k] = (threadIdx.y * ARPT + k + R) * A.spitch + threadIdx.x + R;
      f2 z;
      if (STAGED) z = make_float2(zs[ci[k]], zs[ci[k] + AX]);
      else z = make_float2(load_clamped(A, T, yb + k, xa), load_clamped(A, T, yb + k, xb));
      nz[k] = make_float2(-z.x, -z.y);
      tot[k] = S2(0.f);
      cnt[k] = S2(0.f);
    }
    if (STAGED && !any_nan) {
      // every sample valid: count = number of samples
#pragma unroll 2
      for (int s = 0; s < A.ns; ++s) {
        const int so = soff[s];
        const float r = ss[s].r, df = ss[s].df;
#pragma unroll
        for (int k = 0; k < ARPT; ++k) {
          const f2 v = make_float2(zs[ci[k] + so], zs[ci[k] + so + AX]);
          tot[k] = __ffma2_rn(occlusion2(v, nz[k], r), S2(df), tot[k]);
        }
      }
#pragma unroll
      for (int k = 0; k < ARPT; ++k) cnt[k] = S2((float)A.ns);
    } else {
      for (int s = 0; s < A.ns; ++s) {
        const AoSample smp = ss[s];
        const int so = soff[s];
#pragma unroll
        for (int k = 0; k < ARPT; ++k) {
          f2 v;
          if (STAGED) v = make_float2(zs[ci[k] + so], zs[ci[k] + so + AX]);
          else v = make_float2(load_clamped(A, T, yb + k + smp.oy, xa + smp.ox),
                               load_clamped(A, T, yb + k + smp.oy, xb + smp.ox));
          // np.where(valid, occlusion * factor, 0): an invalid sample's occlusion is 0
          tot[k] = __ffma2_rn(occlusion2(v, nz[k], smp.r), S2(smp.df), tot[k]);
          cnt[k] = __fadd2_rn(cnt[k], make_float2(v.x == v.x ? 1.f : 0.f, v.y == v.y ? 1.f : 0.f));
        }
      }
    }
    float* F = A.field + A.foff[t];
#pragma unroll
    for (int k = 0; k < ARPT; ++k) {
      const int y = yb + k;
      if (y >= E.y0 + E.h) continue;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int x = c ? xb : xa;
        if (x >= E.x0 + E.w) continue;
        const float z = c ? -nz[k].y : -nz[k].x;
        float v = 1.0f;  // NoData cells enter the Gaussian as 1
        if (z == z) {
          const float mean = __fdiv_rn(c ? tot[k].y : tot[k].x, fmaxf(c ? cnt[k].y : cnt[k].x, 1.0f));
          v = fminf(fmaxf(__fsub_rn(1.0f, __fmul_rn(mean, A.intensity)), 0.0f), 1.0f);
        }
        F[(long long)(y - E.y0) * E.w + (x - E.x0)] = v;
      }
    }
  }
}

// scipy's symmetric 9-tap correlate1d (float64 weights and accumulator),
// x[4] w0 + (x[0] + x[8]) w4 + ... + (x[3] + x[5]) w1, rounded to float32.
// Compensated dot product (Ogita, Rump and Oishi's Dot2): each pair sum and
// each product with the weight's high part is split exactly (TwoSum,
// TwoProduct by FMA), the running sum is kept exact by TwoSum, and all
// low-order terms (the splits' errors and the weights' low parts) collect in
// one float32 correction; the result is as accurate as a twice-as-wide
// accumulation rounded once.
__device__ __forceinline__ float gsum9(const FF* w, const float* x) {
  float s = __fmul_rn(x[4], w[0].hi);
  float c = __fmaf_rn(x[4], w[0].hi, -s);
  c = __fmaf_rn(x[4], w[0].lo, c);
#pragma unroll
  for (int k = 4; k >= 1; --k) {
    const FF p = two_sum(x[4 - k], x[4 + k]);
    const float q = __fmul_rn(p.hi, w[k].hi);
    float e = __fmaf_rn(p.hi, w[k].hi, -q);
    e = __fmaf_rn(p.hi, w[k].lo, e);
    e = __fmaf_rn(p.lo, w[k].hi, e);
    const FF t = two_sum(s, q);
    s = t.hi;
    c = __fadd_rn(c, __fadd_rn(t.lo, e));
  }
  return __fadd_rn(s, c);
}

__global__ void __launch_bounds__(AX * AY) ao_finish_kernel(const __grid_constant__ AoArgs A) {
  __shared__ float tz[FTH][FTW];      // field, rows/cols clamped to the field region
  __shared__ float t0[APH][FTW + 1];  // axis-0 pass (float32 intermediate)
  const int tid = threadIdx.y * AX + threadIdx.x;
  FF gw[GR + 1];
#pragma unroll
  for (int j = 0; j <= GR; ++j) gw[j] = A.gw[j];
  const float qnan = __int_as_float(0x7fc00000);
  for (int blk = blockIdx.x; blk < A.out_blocks; blk += gridDim.x) {
    const int t = tile_of(A.oblock0, A.ntiles, blk);
    const fsg_tile T = A.tiles[t];
    const FieldReg E = A.freg[t];
    const int nbx = (T.core_w + APW - 1) / APW;
    const int lb = blk - A.oblock0[t];
    const int by = lb / nbx, bx = lb - by * nbx;
    const int bx0 = T.core_x0 + bx * APW, by0 = T.core_y0 + by * APH;
    const float* F = A.field + A.foff[t];
    __syncthreads();
    for (int i = tid; i < FTH * FTW; i += AX * AY) {
      const int r = i / FTW, c = i - (i / FTW) * FTW;
      const int fy = min(max(by0 - GR + r - E.y0, 0), E.h - 1);
      const int fx = min(max(bx0 - GR + c - E.x0, 0), E.w - 1);
      tz[r][c] = F[(long long)fy * E.w + fx];
    }
    __syncthreads();
    for (int i = tid; i < APH * FTW; i += AX * AY) {
      const int r = i / FTW, c = i - (i / FTW) * FTW;
      float x[9];
#pragma unroll
      for (int j = 0; j < 9; ++j) x[j] = tz[r + j][c];
      t0[r][c] = gsum9(gw, x);
    }
    __syncthreads();
    for (int i = tid; i < APH * APW; i += AX * AY) {
      const int r = i / APW, c = i - (i / APW) * APW;
      const int y = by0 + r, xx = bx0 + c;
      if (y >= T.core_y0 + T.core_h || xx >= T.core_x0 + T.core_w) continue;
      float x[9];
#pragma unroll
      for (int j = 0; j < 9; ++j) x[j] = t0[r][c + j];
      const float g = gsum9(gw, x);
      const float z = __ldg(A.raster + (long long)y * A.ld + xx);
      float v;
      if (is_nodata(z, A.ndf, A.has_nodata != 0)) {
        v = qnan;
      } else {
        v = g > 0.f ? exp2f(0.45454545454545453f * __log2f(g)) : 0.0f;
        if (A.scale > 0.f) v = fmaxf(__fdiv_rn(__fsub_rn(v, A.lo), A.scale), 0.0f);
      }
      const long long o = (long long)(T.out_y0 + (y - T.core_y0)) * A.old + (T.out_x0 + (xx - T.core_x0));
      if (A.odtype == FSG_F32) static_cast<float*>(A.out)[o] = v;
      else if (A.odtype == FSG_U8) static_cast<uint8_t*>(A.out)[o] = (uint8_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
      else static_cast<int16_t*>(A.out)[o] = (int16_t)(int)quantize(v, A.qa, A.qb, A.qmin, A.qmax);
    }
  }
}

// Python's round() / np.round: nearest integer, ties to even.
int round_half_even(double v) { return (int)std::nearbyint(v); }

}  // namespace

// The sample offsets and ring distance factors, ring-major (_impl_ambient_occlusion.py:54-88).
static void ao_offsets(int num_samples, double radius, std::vector<AoSample>* out) {
  out->clear();
  const double rings[4] = {0.25, 0.5, 0.75, 1.0};
  const double step = (2.0 * M_PI) / (double)num_samples;
  for (double rf : rings) {
    const double r = radius * rf;
    const float df = (float)(1.0 - rf * 0.3);
    for (int i = 0; i < num_samples; ++i) {
      const double th = (double)i * step;
      const int ox = round_half_even(r * std::cos(th)), oy = round_half_even(r * std::sin(th));
      if (ox == 0 && oy == 0) continue;
      AoSample s;
      s.ox = (short)ox;
      s.oy = (short)oy;
      s.r = 0.f;
      s.df = df;
      out->push_back(s);
    }
  }
}

// One ambient-occlusion job: the packed device tables (host image), the
// kernel arguments and the launch shapes; the field scratch follows the tables.
struct AoJob {
  bool empty = true;
  std::vector<char> host;
  size_t o_s = 0, o_t = 0, o_fr = 0, o_fo = 0, o_fb = 0, o_ob = 0, o_field = 0;
  size_t field_bytes = 0;
  AoArgs A;
  void (*fieldk)(AoArgs) = nullptr;
  int fgrid = 0, ogrid = 0;
  size_t fsmem = 0;
  size_t device_bytes() const { return o_field + field_bytes; }
  void bind(void* dev) {
    char* base = static_cast<char*>(dev);
    A.samples = reinterpret_cast<const AoSample*>(base + o_s);
    A.tiles = reinterpret_cast<const fsg_tile*>(base + o_t);
    A.freg = reinterpret_cast<const FieldReg*>(base + o_fr);
    A.foff = reinterpret_cast<const long long*>(base + o_fo);
    A.fblock0 = reinterpret_cast<const int*>(base + o_fb);
    A.oblock0 = reinterpret_cast<const int*>(base + o_ob);
    A.field = reinterpret_cast<float*>(base + o_field);
  }
  int upload(void* dev, cudaStream_t s) const {
    FSG_UPLOAD(dev, host.data(), host.size(), s);
    return FSG_OK;
  }
  int enqueue(cudaStream_t s) const {
    if (empty) return FSG_OK;
    timing_mark(s, true);
    fieldk<<<fgrid, dim3(AX, AY), fsmem, s>>>(A);
    timing_mark(s, false);
    FSG_LAUNCHED(1);
    ao_finish_kernel<<<ogrid, dim3(AX, AY), 0, s>>>(A);
    FSG_LAUNCHED(1);
    return FSG_OK;
  }
};

static int ao_prepare(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w, const fsg_tile* tiles,
                      int32_t ntiles, const fsg_ao_params* p, const fsg_plane* out, AoJob& J) {
  if (!p || (ntiles > 0 && !tiles)) return fail(FSG_ERR_INVALID, "null argument");
  if (ntiles < 0 || raster_h < 0 || raster_w < 0 || ld < raster_w) return fail(FSG_ERR_INVALID, "bad raster shape");
  if (!out || !out->ptr) return fail(FSG_ERR_INVALID, "no output plane");
  if (out->dtype < FSG_F32 || out->dtype > FSG_I16) return fail(FSG_ERR_DTYPE, "dtype %d", out->dtype);
  if (p->num_samples < 1 || p->num_samples > 4096 || !(p->radius >= 0.0) || !std::isfinite(p->radius) ||
      p->radius > 16384.0 || !std::isfinite(p->intensity))
    return fail(FSG_ERR_INVALID, "bad ambient occlusion parameters");
  int st = validate_tiles(raster_h, raster_w, tiles, ntiles, 1);
  if (st) return st;
  std::vector<AoSample> offs;
  ao_offsets(p->num_samples, p->radius, &offs);
  const int ns = (int)offs.size();
  int reach = 0;
  for (const AoSample& s : offs) reach = std::max(reach, std::max(std::abs((int)s.ox), std::abs((int)s.oy)));
  std::vector<AoSample> samples;
  samples.reserve((size_t)ns * std::max(ntiles, 1));
  std::vector<FieldReg> freg;
  std::vector<long long> foff;
  std::vector<int> fb0, ob0;
  long long field_elems = 0;
  int fblocks = 0, oblocks = 0;
  for (int t = 0; t < ntiles; ++t) {
    const fsg_tile& T = tiles[t];
    // _impl_ambient_occlusion.py:59-64
    double sx = std::fabs(T.pixel_scale_x), sy = std::fabs(T.pixel_scale_y);
    const double fb = p->pixel_size != 0.0 ? p->pixel_size : 1.0;
    if (sx < 1e-9) sx = fb;
    if (sy < 1e-9) sy = fb;
    for (AoSample s : offs) {
      const double d = std::max(std::hypot((double)s.ox * sx, (double)s.oy * sy), 1e-9);
      s.r = 1.0f / (float)d;
      samples.push_back(s);
    }
    FieldReg e = {0, 0, 0, 0};
    if (T.core_h > 0 && T.core_w > 0) {
      const int y0 = std::max(T.core_y0 - GR, T.win_y0), y1 = std::min(T.core_y0 + T.core_h + GR, T.win_y0 + T.win_h);
      const int x0 = std::max(T.core_x0 - GR, T.win_x0), x1 = std::min(T.core_x0 + T.core_w + GR, T.win_x0 + T.win_w);
      e = {y0, x0, y1 - y0, x1 - x0};
    }
    freg.push_back(e);
    foff.push_back(field_elems);
    field_elems += ((long long)e.h * e.w + 3) & ~3LL;
    fb0.push_back(fblocks);
    ob0.push_back(oblocks);
    if (e.h > 0 && e.w > 0) {
      fblocks += ((e.w + APW - 1) / APW) * ((e.h + APH - 1) / APH);
      oblocks += ((T.core_w + APW - 1) / APW) * ((T.core_h + APH - 1) / APH);
    }
  }
  if (oblocks == 0) {
    J.empty = true;
    return FSG_OK;
  }
  auto al = [](size_t n) { return (n + 255) & ~(size_t)255; };
  const size_t b_s = samples.size() * sizeof(AoSample), b_t = (size_t)ntiles * sizeof(fsg_tile);
  const size_t b_fr = freg.size() * sizeof(FieldReg), b_fo = foff.size() * sizeof(long long);
  const size_t b_fb = fb0.size() * sizeof(int), b_ob = ob0.size() * sizeof(int);
  const size_t bytes = al(b_s) + al(b_t) + al(b_fr) + al(b_fo) + al(b_fb) + al(b_ob);
  J.host.assign(bytes, 0);
  size_t off = 0;
  auto put = [&](const void* src, size_t n) {
    if (n) std::memcpy(J.host.data() + off, src, n);
    const size_t o = off;
    off += al(n);
    return o;
  };
  J.o_s = put(samples.data(), b_s);
  J.o_t = put(tiles, b_t);
  J.o_fr = put(freg.data(), b_fr);
  J.o_fo = put(foff.data(), b_fo);
  J.o_fb = put(fb0.data(), b_fb);
  J.o_ob = put(ob0.data(), b_ob);
  J.o_field = off;
  J.field_bytes = (size_t)field_elems * sizeof(float);
  AoArgs& A = J.A;
  std::memset(&A, 0, sizeof(A));
  A.raster = raster_dev;
  A.ld = ld;
  A.ndf = (float)p->nodata;
  A.has_nodata = p->has_nodata != 0;
  A.ns = ns;
  A.reach = reach;
  A.intensity = (float)p->intensity;
  A.ntiles = ntiles;
  A.field_blocks = fblocks;
  A.out_blocks = oblocks;
  int R = 0;
  const std::vector<FF> g = ff_gaussian(1.0, &R);
  for (int j = 0; j <= GR; ++j) A.gw[j] = g[j];
  A.lo = (float)p->stretch_lo;
  A.scale = p->stretch_scale > 1e-12 ? (float)p->stretch_scale : 0.0f;
  A.out = out->ptr;
  A.old = out->ld;
  A.odtype = out->dtype;
  A.qa = out->q_a;
  A.qb = out->q_b;
  A.qmin = out->q_min;
  A.qmax = out->q_max;
  DeviceInfo di;
  st = device_info(&di);
  if (st) return st;
  const size_t tables = (size_t)ns * sizeof(AoSample) + (size_t)((ns + 3) & ~3) * sizeof(int);
  if (tables > di.smem_optin)
    return fail(FSG_ERR_UNSUPPORTED, "%d samples need %zu B of shared-memory tables (at most %zu)", ns, tables,
                di.smem_optin);
  const int spitch = APW + 2 * reach;
  const size_t staged = tables + sizeof(float) * (size_t)spitch * (APH + 2 * reach);
  if (staged <= di.smem_optin) {
    A.spitch = spitch;
    J.fieldk = ao_field_kernel<true>;
    J.fsmem = staged;
  } else {
    A.spitch = 0;
    J.fieldk = ao_field_kernel<false>;
    J.fsmem = tables;
  }
  if (J.fsmem > 48 * 1024)
    FSG_CUDA(cudaFuncSetAttribute(J.fieldk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)J.fsmem));
  int per_sm = 0;
  FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, J.fieldk, AX * AY, J.fsmem));
  J.fgrid = std::min(fblocks, di.sms * std::max(1, per_sm));
  FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ao_finish_kernel, AX * AY, 0));
  J.ogrid = std::min(oblocks, di.sms * std::max(1, per_sm));
  J.empty = false;
  return FSG_OK;
}

struct AoPlan final : fsg_plan {
  AoJob J;
  void* dev = nullptr;
  ~AoPlan() override {
    if (dev) cudaFree(dev);
  }
  int launch(cudaStream_t s) override { return J.enqueue(s); }
};
}  // namespace fsg

extern "C" int fsg_ambient_occlusion(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                                     const fsg_tile* tiles, int32_t ntiles, const fsg_ao_params* params,
                                     const fsg_plane* out, void* stream) {
  using namespace fsg;
  AoJob J;
  int st = ao_prepare(raster_dev, ld, raster_h, raster_w, tiles, ntiles, params, out, J);
  if (st || J.empty) return st;
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch scratch;
  st = scratch.alloc(J.device_bytes(), s);
  if (st) return st;
  J.bind(scratch.ptr);
  st = J.upload(scratch.ptr, s);
  if (st) return st;
  return J.enqueue(s);
}

extern "C" int fsg_ambient_occlusion_plan(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                                          const fsg_tile* tiles, int32_t ntiles, const fsg_ao_params* params,
                                          const fsg_plane* out, fsg_plan** plan) {
  using namespace fsg;
  if (!plan) return fail(FSG_ERR_INVALID, "null plan pointer");
  *plan = nullptr;
  AoPlan* P = new AoPlan();
  int st = ao_prepare(raster_dev, ld, raster_h, raster_w, tiles, ntiles, params, out, P->J);
  if (!st && !P->J.empty) {
    cudaError_t e = cudaMalloc(&P->dev, P->J.device_bytes());
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
