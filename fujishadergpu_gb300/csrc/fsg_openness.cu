// Topographic openness (Yokoyama et al. 2002), exact ray-march.
//
// Reference semantics (algorithms/_impl_openness.py:31-132), per tile window:
//   directions theta_d = 2*pi*d/n (np.linspace(0, 2pi, n, endpoint=False));
//   sample offsets (int(round(r cos)), int(round(r sin))) with Python's
//   round-half-to-even, (0, 0) skipped, for the distances
//     reference mode: unique(int(linspace(0.1, 1, 10) * D)) > 0   (:65-68)
//     dense mode    : every step r = 1..D (the O(px * dirs * D) ray-march);
//   a sample is valid inside the window and off NoData (:81-83, :112);
//   angle = atan((z_s - z) / hypot(ox*|sx|, oy*|sy|)); per direction the max
//   (positive) / min (negative) over valid samples; directional mean of
//   pi/2 - max (positive) or pi/2 + min (negative) over directions with a
//   valid sample (:119-126); display = clip(mean/(pi/2), 0, 1)^(1/2.2)
//   (:127-129), optionally stretched by global (p1, p99 - p1) stats
//   (algorithms/tile/dask_bridge.py:173-187).
//
// atan is monotonic, so the per-direction extreme angle is atan of the
// extreme slope ratio: each sample costs one load, one subtract, one multiply
// by the rounded reciprocal of its float32 distance (within 1.5 ulp of the
// reference's float32 division; the mean angle's tolerance is 0.01 degree)
// and one max; atan runs once per direction.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fsg_common.cuh"

namespace fsg {
namespace {

constexpr int BX = 32, BY = 8, RPT = 4;  // block 32 x 8 threads; a thread: 4 rows x 2 columns
constexpr int PW = 2 * BX, PH = BY * RPT;  // pixels per block: 64 x 32

struct RaySample {
  short ox, oy;
  float d, r;  // f32(distance), RN(1/d)
};

struct OpenArgs {
  const float* raster;
  long long ld;
  int rh, rw;
  float ndf;
  int has_nodata;
  int positive;
  int ndir;
  int ns;                      // samples per tile (all directions)
  const int* ray_begin;        // [ntiles * (ndir + 1)] offsets into samples
  const RaySample* samples;    // per tile: its own distance table
  const int* tile_sample0;     // first sample index of each tile
  const int* tile_reach;       // per tile: max |ox|, max |oy| of its samples
  const fsg_tile* tiles;       // device copy
  const int* block0;           // first block of each tile
  int ntiles, total_blocks;
  float lo, scale;             // display stretch (scale <= 0: none)
  void* disp;
  long long dld;
  int ddtype;
  float qa, qb;
  int qmin, qmax;
  float* raw;                  // mean angle in degrees (nullable)
  long long rld;
  unsigned* queue;             // work queue: next block of the flattened tile list (zeroed per launch)
};

__device__ __forceinline__ float load_z(const OpenArgs& A, int y, int x, const fsg_tile& T) {
  if (y < T.win_y0 || y >= T.win_y0 + T.win_h || x < T.win_x0 || x >= T.win_x0 + T.win_w)
    return __int_as_float(0x7fc00000);
  float v = __ldg(A.raster + (long long)y * A.ld + x);
  return is_nodata(v, A.ndf, A.has_nodata != 0) ? __int_as_float(0x7fc00000) : v;
}

typedef float2 f2;
__device__ __forceinline__ f2 S2(float a) { return make_float2(a, a); }
// (v - z) / d per component as (v - z) * RN(1/d); nz = -z
__device__ __forceinline__ f2 slope2(f2 v, f2 nz, float r) {
  return __fmul2_rn(__fadd2_rn(v, nz), S2(r));
}
__device__ __forceinline__ float nd_nan(float v, const OpenArgs& A) {
  return is_nodata(v, A.ndf, true) ? __int_as_float(0x7fc00000) : v;
}

// Per pixel pair (x, x+1) and row: the per-direction extreme slope ratio of
// the valid samples (NaN samples drop out: fmaxf / fminf return the other
// operand), atan of it once per direction, directional mean.  Blocks whose
// rays stay inside the window (all but the window's outer ring) take the
// interior path: one element offset per sample, no bounds checks.
// IDX32: the raster holds fewer than 2^32 elements, so the interior path
// addresses samples with 32-bit element indices from the raster base.
#ifndef FSG_OPEN_MINB
#define FSG_OPEN_MINB 4  // resident blocks per SM the register budget must allow (occupancy hides the gathers)
#endif
// UNR: samples per iteration of the interior sample loop (their gathers in flight
// together): 2 for the reference sampling (10 samples per ray; 3.6 % faster at
// 16384^2 than 1), 1 for the dense ray-march (2 measured 2 % slower there).
template <bool POS, bool HN, bool IDX32, int UNR>
__global__ void __launch_bounds__(BX * BY, FSG_OPEN_MINB) openness_kernel(const __grid_constant__ OpenArgs A) {
  extern __shared__ unsigned char osm[];
  int* soff = reinterpret_cast<int*>(osm);             // [ns] element offset oy * ld + ox
  float* sd = reinterpret_cast<float*>(soff + A.ns);   // [ns] distance
  float* sr = sd + A.ns;                               // [ns] RN(1/d)
  short* sox = reinterpret_cast<short*>(sr + A.ns);    // [ns]
  short* soy = sox + A.ns;                             // [ns]
  const int tid = threadIdx.y * BX + threadIdx.x;
  int loaded = -1;
  const float init = POS ? -INFINITY : INFINITY;
  const float half_pi = 1.57079637050628662109375f;  // f32(pi/2)
  // Blocks of all tiles (of any size and overview level) are popped from one device
  // queue, so CTAs that draw cheap blocks take more of them.  The pop is uniform
  // over the CTA (thread 0 draws, a barrier publishes it).
  __shared__ int s_blk;
  auto pop = [&]() -> int {
    __syncthreads();
    if (tid == 0) s_blk = (int)atomicAdd(A.queue, 1u);
    __syncthreads();
    return s_blk;
  };
  for (int blk = pop(); blk < A.total_blocks; blk = pop()) {
    int lo = 0, hi = A.ntiles - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (A.block0[mid] <= blk) lo = mid; else hi = mid - 1;
    }
    const fsg_tile T = A.tiles[lo];
    if (lo != loaded) {  // stage this tile's sample table
      __syncthreads();
      const RaySample* S = A.samples + A.tile_sample0[lo];
      for (int i = tid; i < A.ns; i += BX * BY) {
        const RaySample rs = S[i];
        soff[i] = (int)rs.oy * (int)A.ld + (int)rs.ox;
        sd[i] = rs.d;
        sr[i] = rs.r;
        sox[i] = rs.ox;
        soy[i] = rs.oy;
      }
      loaded = lo;
      __syncthreads();
    }
    const int* rb = A.ray_begin + lo * (A.ndir + 1);
    const int nbx = (T.core_w + PW - 1) / PW;
    const int lb = blk - A.block0[lo];
    const int by = lb / nbx, bx = lb - by * nbx;
    const int bx0 = T.core_x0 + bx * PW, by0 = T.core_y0 + by * PH;
    const int x = bx0 + 2 * threadIdx.x;
    const int yb = by0 + threadIdx.y * RPT;
    const int rx = A.tile_reach[2 * lo], ry = A.tile_reach[2 * lo + 1];
    const bool interior = bx0 - rx >= T.win_x0 && bx0 + PW + rx <= T.win_x0 + T.win_w && by0 - ry >= T.win_y0 &&
                          by0 + PH + ry <= T.win_y0 + T.win_h;
    const bool cx0 = x < T.core_x0 + T.core_w, cx1 = x + 1 < T.core_x0 + T.core_w;
    f2 z[RPT], sum[RPT], cnt[RPT];
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const bool row = yb + k < T.core_y0 + T.core_h;
      z[k].x = (row && cx0) ? load_z(A, yb + k, x, T) : __int_as_float(0x7fc00000);
      z[k].y = (row && cx1) ? load_z(A, yb + k, x + 1, T) : __int_as_float(0x7fc00000);
      sum[k] = S2(0.f);
      cnt[k] = S2(0.f);
    }
    const float* base = A.raster + (long long)yb * A.ld + x;
    const unsigned idx0 = IDX32 ? (unsigned)((long long)yb * A.ld + x) : 0u;
    // x is even and the raster base and row pitch keep even elements 8-byte aligned
    const bool pair_ok = ((x & 1) == 0) && ((A.ld & 1) == 0) && ((reinterpret_cast<uintptr_t>(A.raster) & 7) == 0);
    f2 nz[RPT];
#pragma unroll
    for (int k = 0; k < RPT; ++k) nz[k] = make_float2(-z[k].x, -z[k].y);
    for (int d = 0; d < A.ndir; ++d) {
      f2 ext[RPT];
#pragma unroll
      for (int k = 0; k < RPT; ++k) ext[k] = S2(init);
      if (interior) {
#pragma unroll UNR
        for (int s = rb[d]; s < rb[d + 1]; ++s) {
          const int so = soff[s];
          const float rr = sr[s];
          // the pixel pair's sample pair is 8-byte aligned when the offset is even (uniform per sample)
          const bool pair = pair_ok && (so & 1) == 0;
#pragma unroll
          for (int k = 0; k < RPT; ++k) {
            const float* pk;
            if (IDX32) pk = A.raster + (unsigned)(idx0 + (unsigned)k * (unsigned)A.ld + (unsigned)so);
            else pk = base + (long long)k * A.ld + so;
            f2 v;
            if (pair) v = __ldg(reinterpret_cast<const float2*>(pk));
            else v = make_float2(__ldg(pk), __ldg(pk + 1));
            if (HN) v = make_float2(nd_nan(v.x, A), nd_nan(v.y, A));
            const f2 t = slope2(v, nz[k], rr);
            ext[k].x = POS ? fmaxf(ext[k].x, t.x) : fminf(ext[k].x, t.x);
            ext[k].y = POS ? fmaxf(ext[k].y, t.y) : fminf(ext[k].y, t.y);
          }
        }
      } else {
        for (int s = rb[d]; s < rb[d + 1]; ++s) {
          const int ox = sox[s], oy = soy[s];
          const float rr = sr[s];
#pragma unroll
          for (int k = 0; k < RPT; ++k) {
            const f2 v = make_float2(load_z(A, yb + k + oy, x + ox, T), load_z(A, yb + k + oy, x + 1 + ox, T));
            const f2 t = slope2(v, nz[k], rr);
            ext[k].x = POS ? fmaxf(ext[k].x, t.x) : fminf(ext[k].x, t.x);
            ext[k].y = POS ? fmaxf(ext[k].y, t.y) : fminf(ext[k].y, t.y);
          }
        }
      }
#pragma unroll
      for (int k = 0; k < RPT; ++k) {
        // atan of the extreme ratio once per direction; directions without a valid sample drop out
        if (ext[k].x != init) {
          const float a = atanf(ext[k].x);
          sum[k].x = __fadd_rn(sum[k].x, POS ? __fsub_rn(half_pi, a) : __fadd_rn(half_pi, a));
          cnt[k].x = __fadd_rn(cnt[k].x, 1.0f);
        }
        if (ext[k].y != init) {
          const float a = atanf(ext[k].y);
          sum[k].y = __fadd_rn(sum[k].y, POS ? __fsub_rn(half_pi, a) : __fadd_rn(half_pi, a));
          cnt[k].y = __fadd_rn(cnt[k].y, 1.0f);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int y = yb + k;
      if (y >= T.core_y0 + T.core_h) continue;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int xx = x + c;
        if (xx >= T.core_x0 + T.core_w) continue;
        const float zz = c ? z[k].y : z[k].x;
        const float sm = c ? sum[k].y : sum[k].x, cn = c ? cnt[k].y : cnt[k].x;
        float mean = __fdiv_rn(sm, fmaxf(cn, 1.0f));
        float disp, rawd;
        if (zz != zz) {
          disp = rawd = __int_as_float(0x7fc00000);
        } else {
          float op = fminf(fmaxf(__fdiv_rn(mean, half_pi), 0.0f), 1.0f);
          disp = op > 0.f ? exp2f(0.45454545454545453f * __log2f(op)) : 0.0f;
          if (A.scale > 0.f) disp = fmaxf(__fdiv_rn(__fsub_rn(disp, A.lo), A.scale), 0.0f);
          rawd = mean * 57.295780181884765625f;
        }
        const long long py = T.out_y0 + (y - T.core_y0), px = T.out_x0 + (xx - T.core_x0);
        if (A.disp) {
          long long o = py * A.dld + px;
          if (A.ddtype == FSG_F32) static_cast<float*>(A.disp)[o] = disp;
          else if (A.ddtype == FSG_U8) static_cast<uint8_t*>(A.disp)[o] = (uint8_t)(int)quantize(disp, A.qa, A.qb, A.qmin, A.qmax);
          else static_cast<int16_t*>(A.disp)[o] = (int16_t)(int)quantize(disp, A.qa, A.qb, A.qmin, A.qmax);
        }
        if (A.raw) A.raw[py * A.rld + px] = rawd;
      }
    }
  }
}

}  // namespace

// Python's round(): nearest integer, ties to even.
static int py_round(double v) { return (int)std::nearbyint(v); }

// Ray offsets in pixels: per direction a list of (ox, oy).
static void ray_offsets(int ndir, int max_distance, int mode, std::vector<std::vector<std::pair<int, int>>>* out) {
  std::vector<int> dist;
  if (mode == 0) {
    // np.unique((np.linspace(0.1, 1.0, 10) * D).astype(int)), > 0
    for (int i = 0; i < 10; ++i) {
      double t = 0.1 + (double)i * ((1.0 - 0.1) / 9.0);
      if (i == 9) t = 1.0;
      dist.push_back((int)(t * (double)max_distance));
    }
    std::sort(dist.begin(), dist.end());
    dist.erase(std::unique(dist.begin(), dist.end()), dist.end());
    dist.erase(std::remove_if(dist.begin(), dist.end(), [](int r) { return r <= 0; }), dist.end());
  } else {
    for (int r = 1; r <= max_distance; ++r) dist.push_back(r);
  }
  out->assign(ndir, {});
  const double step = (2.0 * M_PI) / (double)ndir;
  for (int d = 0; d < ndir; ++d) {
    double th = (double)d * step;
    double c = std::cos(th), s = std::sin(th);
    for (int r : dist) {
      int ox = py_round((double)r * c), oy = py_round((double)r * s);
      if (ox == 0 && oy == 0) continue;
      (*out)[d].push_back({ox, oy});
    }
  }
}

}  // namespace fsg

using namespace fsg;

extern "C" int fsg_openness_offsets(int32_t num_directions, int32_t max_distance, int32_t mode, int32_t* ox,
                                    int32_t* oy, int32_t* ray_len, int32_t capacity) {
  if (num_directions < 1 || max_distance < 0 || mode < 0 || mode > 1 || !ray_len)
    return fail(FSG_ERR_INVALID, "bad openness ray parameters");
  std::vector<std::vector<std::pair<int, int>>> rays;
  ray_offsets(num_directions, max_distance, mode, &rays);
  int n = 0;
  for (int d = 0; d < num_directions; ++d) {
    ray_len[d] = (int32_t)rays[d].size();
    for (auto& o : rays[d]) {
      if (n < capacity && ox && oy) {
        ox[n] = o.first;
        oy[n] = o.second;
      }
      ++n;
    }
  }
  if (n > capacity) return fail(FSG_ERR_WORKSPACE, "need %d offset slots, have %d", n, capacity);
  return FSG_OK;
}

namespace fsg {
// One openness job: the packed device tables (host image), the kernel
// arguments and the launch shape.  The eager entry point uploads the image
// into stream-ordered scratch; a plan uploads it once into memory it owns.
struct OpenJob {
  bool empty = true;
  std::vector<char> host;
  size_t o_s = 0, o_rb = 0, o_ts = 0, o_b0 = 0, o_t = 0, o_re = 0, o_q = 0;
  OpenArgs A;
  void (*kern)(OpenArgs) = nullptr;
  int grid = 0;
  size_t smem = 0;
  void bind(void* dev) {
    char* base = static_cast<char*>(dev);
    A.tile_reach = reinterpret_cast<const int*>(base + o_re);
    A.samples = reinterpret_cast<const RaySample*>(base + o_s);
    A.ray_begin = reinterpret_cast<const int*>(base + o_rb);
    A.tile_sample0 = reinterpret_cast<const int*>(base + o_ts);
    A.block0 = reinterpret_cast<const int*>(base + o_b0);
    A.tiles = reinterpret_cast<const fsg_tile*>(base + o_t);
    A.queue = reinterpret_cast<unsigned*>(base + o_q);
  }
  int upload(void* dev, cudaStream_t s) const {
    FSG_UPLOAD(dev, host.data(), host.size(), s);
    return FSG_OK;
  }
  int enqueue(cudaStream_t s) const {
    if (empty) return FSG_OK;
    FSG_CUDA(cudaMemsetAsync(A.queue, 0, sizeof(unsigned), s));
    timing_mark(s, true);
    kern<<<grid, dim3(BX, BY), smem, s>>>(A);
    timing_mark(s, false);
    FSG_LAUNCHED(1);
    return FSG_OK;
  }
};

static int openness_prepare(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                            const fsg_tile* tiles, int32_t ntiles, const fsg_openness_params* p,
                            const fsg_plane* display, float* raw_deg_dev, int64_t raw_ld, OpenJob& J) {
  if (!p || (ntiles > 0 && !tiles)) return fail(FSG_ERR_INVALID, "null argument");
  if (ntiles < 0 || raster_h < 0 || raster_w < 0 || ld < raster_w) return fail(FSG_ERR_INVALID, "bad raster shape");
  if ((!display || !display->ptr) && !raw_deg_dev) return fail(FSG_ERR_INVALID, "no output requested");
  if (display && display->ptr && (display->dtype < FSG_F32 || display->dtype > FSG_I16))
    return fail(FSG_ERR_DTYPE, "dtype %d", display->dtype);
  if (p->num_directions < 1 || p->num_directions > 4096 || p->max_distance < 0 || p->mode < 0 || p->mode > 1)
    return fail(FSG_ERR_INVALID, "bad openness parameters");
  int st = validate_tiles(raster_h, raster_w, tiles, ntiles, 1);
  if (st) return st;
  std::vector<std::vector<std::pair<int, int>>> rays;
  ray_offsets(p->num_directions, p->max_distance, p->mode, &rays);
  const int ndir = p->num_directions;
  int per_tile = 0;
  for (auto& r : rays) per_tile += (int)r.size();
  // Host tables: per tile its distance table (pixel scales may differ per tile).
  std::vector<RaySample> samples;
  std::vector<int> ray_begin, tile_sample0, block0, reach;
  samples.reserve((size_t)per_tile * ntiles);
  int total = 0;
  for (int t = 0; t < ntiles; ++t) {
    const fsg_tile& T = tiles[t];
    // _impl_openness.py:70-75
    double sx = std::fabs(T.pixel_scale_x), sy = std::fabs(T.pixel_scale_y);
    double fb = p->pixel_size != 0.0 ? p->pixel_size : 1.0;
    if (sx < 1e-9) sx = fb;
    if (sy < 1e-9) sy = fb;
    tile_sample0.push_back((int)samples.size());
    int acc = 0, rx = 0, ry = 0;
    for (int d = 0; d < ndir; ++d) {
      ray_begin.push_back(acc);
      for (auto& o : rays[d]) {
        double dist = std::max(std::hypot((double)o.first * sx, (double)o.second * sy), 1e-9);
        RaySample rs;
        rs.ox = (short)o.first;
        rs.oy = (short)o.second;
        rs.d = (float)dist;
        rs.r = 1.0f / rs.d;
        samples.push_back(rs);
        rx = std::max(rx, std::abs(o.first));
        ry = std::max(ry, std::abs(o.second));
        ++acc;
      }
    }
    ray_begin.push_back(acc);
    reach.push_back(rx);
    reach.push_back(ry);
    block0.push_back(total);
    if (T.core_h > 0 && T.core_w > 0) total += ((T.core_w + PW - 1) / PW) * ((T.core_h + PH - 1) / PH);
  }
  J.empty = total == 0;
  if (J.empty) return FSG_OK;
  size_t b_samples = samples.size() * sizeof(RaySample), b_rb = ray_begin.size() * sizeof(int);
  size_t b_ts = tile_sample0.size() * sizeof(int), b_b0 = block0.size() * sizeof(int);
  size_t b_re = reach.size() * sizeof(int);
  size_t b_tiles = (size_t)ntiles * sizeof(fsg_tile);
  auto al = [](size_t n) { return (n + 255) & ~(size_t)255; };
  size_t bytes = al(b_samples) + al(b_rb) + al(b_ts) + al(b_b0) + al(b_tiles) + al(b_re) + al(sizeof(unsigned));
  std::vector<char>& host = J.host;
  host.assign(bytes, 0);
  size_t off = 0;
  auto put = [&](const void* src, size_t n) {
    std::memcpy(host.data() + off, src, n);
    size_t o = off;
    off += al(n);
    return o;
  };
  J.o_s = put(samples.data(), b_samples);
  J.o_rb = put(ray_begin.data(), b_rb);
  J.o_ts = put(tile_sample0.data(), b_ts);
  J.o_b0 = put(block0.data(), b_b0);
  J.o_t = put(tiles, b_tiles);
  J.o_re = put(reach.data(), b_re);
  const unsigned qzero = 0u;
  J.o_q = put(&qzero, sizeof(unsigned));  // the work queue's head
  OpenArgs& A = J.A;
  std::memset(&A, 0, sizeof(A));
  A.raster = raster_dev;
  A.ld = ld;
  A.rh = raster_h;
  A.rw = raster_w;
  A.ndf = (float)p->nodata;
  A.has_nodata = p->has_nodata != 0;
  A.positive = p->openness_type == 0;
  A.ndir = ndir;
  A.ns = per_tile;
  A.ntiles = ntiles;
  A.total_blocks = total;
  A.lo = (float)p->stretch_lo;
  A.scale = p->stretch_scale > 1e-12 ? (float)p->stretch_scale : 0.0f;
  if (display && display->ptr) {
    A.disp = display->ptr;
    A.dld = display->ld;
    A.ddtype = display->dtype;
    A.qa = display->q_a;
    A.qb = display->q_b;
    A.qmin = display->q_min;
    A.qmax = display->q_max;
  }
  A.raw = raw_deg_dev;
  A.rld = raw_ld;
  DeviceInfo di;
  st = device_info(&di);
  if (st) return st;
  if ((long long)p->max_distance * ld >= (1LL << 31))
    return fail(FSG_ERR_UNSUPPORTED, "max_distance %d x row pitch %lld exceeds 32-bit offsets", p->max_distance,
                (long long)ld);
  const bool idx32 = (unsigned long long)ld * (unsigned long long)raster_h < (1ull << 32);
  void (*kern)(OpenArgs) = nullptr;
  if (p->mode == FSG_OPENNESS_DENSE) {
    if (idx32)
      kern = A.positive ? (A.has_nodata ? openness_kernel<true, true, true, 1> : openness_kernel<true, false, true, 1>)
                        : (A.has_nodata ? openness_kernel<false, true, true, 1> : openness_kernel<false, false, true, 1>);
    else
      kern = A.positive ? (A.has_nodata ? openness_kernel<true, true, false, 1> : openness_kernel<true, false, false, 1>)
                        : (A.has_nodata ? openness_kernel<false, true, false, 1> : openness_kernel<false, false, false, 1>);
  } else {
    if (idx32)
      kern = A.positive ? (A.has_nodata ? openness_kernel<true, true, true, 2> : openness_kernel<true, false, true, 2>)
                        : (A.has_nodata ? openness_kernel<false, true, true, 2> : openness_kernel<false, false, true, 2>);
    else
      kern = A.positive ? (A.has_nodata ? openness_kernel<true, true, false, 2> : openness_kernel<true, false, false, 2>)
                        : (A.has_nodata ? openness_kernel<false, true, false, 2> : openness_kernel<false, false, false, 2>);
  }
  const size_t smem = (size_t)per_tile * (3 * sizeof(float) + 2 * sizeof(short)) + 16;
  if (smem > 48 * 1024) FSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  FSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BX * BY, smem));
  J.kern = kern;
  J.smem = smem;
  J.grid = std::min(total, di.sms * std::max(1, per_sm));
  return FSG_OK;
}

struct OpenPlan final : fsg_plan {
  OpenJob J;
  void* dev = nullptr;
  ~OpenPlan() override {
    if (dev) cudaFree(dev);
  }
  int launch(cudaStream_t s) override { return J.enqueue(s); }
};
}  // namespace fsg

extern "C" int fsg_openness(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                            const fsg_tile* tiles, int32_t ntiles, const fsg_openness_params* p,
                            const fsg_plane* display, float* raw_deg_dev, int64_t raw_ld, void* stream) {
  using namespace fsg;
  OpenJob J;
  int st = openness_prepare(raster_dev, ld, raster_h, raster_w, tiles, ntiles, p, display, raw_deg_dev, raw_ld, J);
  if (st || J.empty) return st;
  cudaStream_t s = (cudaStream_t)stream;
  StreamScratch scratch;
  st = scratch.alloc(J.host.size(), s);
  if (st) return st;
  J.bind(scratch.ptr);
  st = J.upload(scratch.ptr, s);
  if (st) return st;
  return J.enqueue(s);
}

extern "C" int fsg_openness_plan(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                                 const fsg_tile* tiles, int32_t ntiles, const fsg_openness_params* p,
                                 const fsg_plane* display, float* raw_deg_dev, int64_t raw_ld, fsg_plan** plan) {
  using namespace fsg;
  if (!plan) return fail(FSG_ERR_INVALID, "null plan pointer");
  *plan = nullptr;
  OpenPlan* P = new OpenPlan();
  int st = openness_prepare(raster_dev, ld, raster_h, raster_w, tiles, ntiles, p, display, raw_deg_dev, raw_ld, P->J);
  if (!st && !P->J.empty) {
    cudaError_t e = cudaMalloc(&P->dev, P->J.host.size());
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
