// Shared helpers of libfsg.so: error reporting, launch accounting, device
// properties and the exactly-rounded float32 primitives the kernels use to
// reproduce NumPy's float32 operation order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "fsg.h"

// A prepared launch (fsg_plan in include/fsg.h): owns the device tables of one
// entry point's call; launch() issues only kernels, memsets and device-side
// copies, so it can be captured in a CUDA graph.
struct fsg_plan {
  virtual ~fsg_plan() {}
  virtual int launch(cudaStream_t s) = 0;
};

namespace fsg {

// ------------------------------------------------------------------ errors
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
void count_launches(int64_t n);
// Records a CUDA event on s around a marked kernel (start before the launch,
// end after it) while fsg_timing_begin is active; no-op otherwise.
void timing_mark(cudaStream_t s, bool start);

#define FSG_CUDA(call)                                      \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return ::fsg::cuda_fail(e_, #call); \
  } while (0)

// Checks the launch that was just queued.
#define FSG_LAUNCHED(n)                                     \
  do {                                                      \
    cudaError_t e_ = cudaGetLastError();                    \
    if (e_ != cudaSuccess) return ::fsg::cuda_fail(e_, "kernel launch"); \
    ::fsg::count_launches(n);                               \
  } while (0)

struct DeviceInfo {
  int device = -1;
  int sms = 0;
  size_t smem_optin = 0;
  size_t smem_per_sm = 0;
};
// Properties of the current device (cached per device).
int device_info(DeviceInfo* out);

// Reads and clears the tensor-core topousm kernel's error word (fsg_topousm_tc.cu).
int tc_take_errors(unsigned* flags);

// Checks a tile list against a raster (windows inside, cores inside windows,
// windows at least `min_window` px on each axis).
int validate_tiles(int32_t raster_h, int32_t raster_w, const fsg_tile* tiles, int32_t ntiles,
                   int min_window);

// The library's stream-ordered memory pool of the current device (kept across calls).
int scratch_pool(cudaMemPool_t* out);

// cudaMemcpyAsync(dst, src, bytes, host to device, s) for a call's tables in pageable
// host memory (copied into pinned staging first, so the call does not wait for the
// work already queued on s).
int upload_async(void* dst, const void* src, size_t bytes, cudaStream_t s);
#define FSG_UPLOAD(dst, src, bytes, s)                             \
  do {                                                             \
    const int st_ = ::fsg::upload_async((dst), (src), (bytes), (s)); \
    if (st_) return st_;                                           \
  } while (0)

// Stream-ordered scratch from the library's pool on `stream`, freed with
// cudaFreeAsync on the same stream by the destructor.
struct StreamScratch {
  void* ptr = nullptr;
  cudaStream_t stream = nullptr;
  StreamScratch() = default;
  StreamScratch(const StreamScratch&) = delete;
  StreamScratch& operator=(const StreamScratch&) = delete;
  int alloc(size_t bytes, cudaStream_t s) {
    stream = s;
    cudaMemPool_t pool = nullptr;
    int st = scratch_pool(&pool);
    if (st) return st;
    cudaError_t e = cudaMallocFromPoolAsync(&ptr, bytes ? bytes : 1, pool, s);
    if (e != cudaSuccess) {
      ptr = nullptr;
      return cuda_fail(e, "cudaMallocFromPoolAsync(scratch)");
    }
    return FSG_OK;
  }
  ~StreamScratch() {
    if (ptr) cudaFreeAsync(ptr, stream);
  }
};

// --------------------------------------------------------- device numerics
// Float32 operations that the compiler may not contract into FMAs: NumPy
// evaluates `a*b + c` on float32 arrays as two separately rounded ufuncs.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// a / d for a divisor d fixed per launch, correctly rounded: q = RN(a*r) with
// r = RN(1/d), then one residual correction q + RN(a - q*d)*r computed with
// fused multiply-adds (P. Markstein, "Computation of elementary functions on
// the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990).  Tested
// against IEEE division on the GPU (tests/test_gpu_numerics.py).
__device__ __forceinline__ float div_by(float a, float d, float r) {
  float q = __fmul_rn(a, r);
  float e = __fmaf_rn(-q, d, a);
  return __fmaf_rn(e, r, q);
}

__device__ __forceinline__ bool is_nodata(float v, float ndf, bool has_nodata) {
  // core/tile_processor.py:185-196 with NumPy 2 scalar rules: the Python
  // float sentinel is applied as a float32 ("weak") scalar.
  if (v != v) return true;
  if (!has_nodata) return false;
  return fabsf(__fsub_rn(v, ndf)) <= 1e-6f || v == ndf;
}

// io/output_encoding.py:178-190: DN = clip(rint(f32(a)*v + f32(b)), lo, hi),
// non-finite -> 0.  Two separately rounded float32 ops, as NumPy does.
__device__ __forceinline__ float quantize(float v, float qa, float qb, int qmin, int qmax) {
  if (!isfinite(v)) return 0.0f;
  float dn = rintf(__fadd_rn(__fmul_rn(qa, v), qb));
  return fminf(fmaxf(dn, (float)qmin), (float)qmax);
}

// The same code without the conversion pipe (rintf and the float -> int cast
// are quarter-rate instructions): the value is clamped first (clamping to
// integer bounds commutes with rint) and then added to 1.5 * 2^23, where the
// spacing of float32 is 1, so the sum's round-to-nearest-even is
// 1.5 * 2^23 + rint(value) and its bit pattern is 0x4B400000 + rint(value) for
// |value| < 2^22.  Returns that bit pattern: its low 8 bits are the uint8 code,
// its low 16 bits the int16 code (two's complement); non-finite -> code 0.
__device__ __forceinline__ uint32_t quantize_bits(float v, float qa, float qb, float fmin, float fmax) {
  float x = fminf(fmaxf(__fadd_rn(__fmul_rn(qa, v), qb), fmin), fmax);
  x = isfinite(v) ? x : 0.0f;
  return __float_as_uint(__fadd_rn(x, 12582912.0f));
}

// ---------------------------------------------------- fast transcendentals
// Float-float ("double-single") arithmetic on the FP32 pipes: a value is
// hi + lo with |lo| <= ulp(hi)/2, about 48 significant bits.  Used for the
// Gaussian filters, which scipy evaluates in float64: the float-float sum
// rounds to the same float32 as scipy's float64 sum except when the exact value
// lies within ~2^-44 (relative) of a float32 rounding boundary.  (GB300's FP64
// rate is a small fraction of its FP32 rate.)
struct FF {
  float hi, lo;
};
// scipy.ndimage._gaussian_kernel1d(sigma, 0, int(4 sigma + 0.5)) normalised in
// float64, as float-float pairs [0..R] (0 = centre).
inline std::vector<FF> ff_gaussian(double sigma, int* radius) {
  const int R = (int)(4.0 * sigma + 0.5);
  std::vector<double> phi(2 * R + 1);
  const double c = -0.5 / (sigma * sigma);
  double s = 0.0;
  for (int k = -R; k <= R; ++k) {
    phi[k + R] = std::exp(c * (double)((long long)k * k));
    s += phi[k + R];
  }
  std::vector<FF> g(R + 1);
  for (int k = 0; k <= R; ++k) {
    const double v = phi[k + R] / s;
    g[k].hi = (float)v;
    g[k].lo = (float)(v - (double)g[k].hi);
  }
  *radius = R;
  return g;
}
__device__ __forceinline__ FF two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ FF fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  FF s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

// Float-float arithmetic on pairs of independent values (the paired FP32
// instructions: per component the same correctly rounded operation as the
// scalar form, so the same results).  The products that a later addition
// consumes are scalar __fmul_rn, which the compiler never contracts into a
// fused multiply-add (a paired multiply followed by a paired add was seen
// fused); the fused multiply-adds of the error terms are intended.
struct FF2 {
  float2 hi, lo;
};
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 p_mul_nc(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
__device__ __forceinline__ FF2 two_sum2(float2 a, float2 b) {
  const float2 s = p_add(a, b), bb = p_sub(s, a);
  return {s, p_add(p_sub(a, p_sub(s, bb)), p_sub(b, bb))};
}
__device__ __forceinline__ FF2 fast_two_sum2(float2 a, float2 b) {
  const float2 s = p_add(a, b);
  return {s, p_sub(b, p_sub(s, a))};
}
__device__ __forceinline__ FF2 ff_mul2(FF2 a, float2 ghi, float2 glo) {  // as ff_mul(a, g) per component
  const float2 p = p_mul_nc(a.hi, ghi);
  float2 e = __ffma2_rn(a.hi, ghi, make_float2(-p.x, -p.y));
  e = __ffma2_rn(a.hi, glo, e);
  e = __ffma2_rn(a.lo, ghi, e);
  return fast_two_sum2(p, e);
}
__device__ __forceinline__ FF2 ff_add2(FF2 a, FF2 b) {  // as ff_add per component
  const FF2 s = two_sum2(a.hi, b.hi);
  return fast_two_sum2(s.hi, p_add(s.lo, p_add(a.lo, b.lo)));
}
__device__ __forceinline__ FF2 ff_scale2(float2 x, float2 ghi, float2 glo) {  // x (hi + lo) per component
  const float2 p = p_mul_nc(x, ghi);
  float2 e = __ffma2_rn(x, ghi, make_float2(-p.x, -p.y));
  e = __ffma2_rn(x, glo, e);
  return fast_two_sum2(p, e);
}

// Hardware approximations (PTX *.approx instructions): relative error ~2^-22.
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// arctan with |error| <= 1.5e-7 rad: atan(a) = a * P(a^2) on [0, 1], P of
// degree 7 fitted to atan(a)/a by iteratively reweighted least squares
// (Lawson's algorithm) on Chebyshev-distributed nodes, and
// atan(x) = pi/2 - atan(1/x) for |x| > 1.
__device__ __forceinline__ float atan_poly(float x) {
  float ax = fabsf(x);
  bool inv = ax > 1.0f;
  float a = inv ? rcp_approx(ax) : ax;
  float a2 = a * a;
  float p = -0x1.09b3ep-8f;
  p = fmaf(a2, p, 0x1.662f9cp-6f);
  p = fmaf(a2, p, -0x1.ca055ep-5f);
  p = fmaf(a2, p, 0x1.8af07cp-4f);
  p = fmaf(a2, p, -0x1.1cd902p-3f);
  p = fmaf(a2, p, 0x1.988166p-3f);
  p = fmaf(a2, p, -0x1.554c3ap-2f);
  p = fmaf(a2, p, 0x1.ffffeap-1f);
  float r = a * p;
  if (inv) r = 1.57079632679489661923f - r;
  return copysignf(r, x);
}
// atan_poly's polynomial for a pair of arguments in [0, 1] (paired FP32 FMAs).
__device__ __forceinline__ float2 atan01_pair(float2 a) {
  auto c = [](float v) { return make_float2(v, v); };
  const float2 a2 = __fmul2_rn(a, a);
  float2 p = c(-0x1.09b3ep-8f);
  p = __ffma2_rn(a2, p, c(0x1.662f9cp-6f));
  p = __ffma2_rn(a2, p, c(-0x1.ca055ep-5f));
  p = __ffma2_rn(a2, p, c(0x1.8af07cp-4f));
  p = __ffma2_rn(a2, p, c(-0x1.1cd902p-3f));
  p = __ffma2_rn(a2, p, c(0x1.988166p-3f));
  p = __ffma2_rn(a2, p, c(-0x1.554c3ap-2f));
  p = __ffma2_rn(a2, p, c(0x1.ffffeap-1f));
  return __fmul2_rn(a, p);
}

}  // namespace fsg
