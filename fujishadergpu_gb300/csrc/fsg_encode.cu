// Elementwise normalisation and output encoding of a float32 plane:
//   v' = (v - offset) / scale             (float32 ops, NaN kept)
//   v' = max(v', 0) when clamp_min0        (display stretch)
//   then float32 store or int16/uint8 code (io/output_encoding.py:178-190).
// Covers apply_global_normalization with topousm_fast_norm_func
// (_global_stats.py:123-153, _normalization.py:35-41: offset 0, scale p99) and
// the openness display stretch (algorithms/tile/dask_bridge.py:173-187:
// offset p1, scale p99 - p1, clamp at 0).
#include "fsg_common.cuh"

namespace fsg {
namespace {
__global__ void affine_kernel(const float* __restrict__ in, long long ld, int h, int w, float off, float sc,
                              int do_scale, int clamp0, void* out, long long old, int dtype, float qa, float qb,
                              int qmin, int qmax) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  for (int y = blockIdx.y * blockDim.y + threadIdx.y; y < h; y += gridDim.y * blockDim.y) {
    if (x >= w) return;
    float v = __ldg(in + (long long)y * ld + x);
    if (do_scale) v = __fdiv_rn(__fsub_rn(v, off), sc);
    if (clamp0 && v == v) v = fmaxf(v, 0.0f);
    long long o = (long long)y * old + x;
    if (dtype == FSG_F32) static_cast<float*>(out)[o] = v;
    else if (dtype == FSG_U8) static_cast<uint8_t*>(out)[o] = (uint8_t)(int)quantize(v, qa, qb, qmin, qmax);
    else static_cast<int16_t*>(out)[o] = (int16_t)(int)quantize(v, qa, qb, qmin, qmax);
  }
}
}  // namespace
}  // namespace fsg

using namespace fsg;

extern "C" int fsg_affine(const float* in_dev, int64_t ld, int32_t h, int32_t w, double offset, double scale,
                          int32_t clamp_min0, const fsg_plane* out, void* stream) {
  if (!in_dev || !out || !out->ptr) return fail(FSG_ERR_INVALID, "null argument");
  if (h < 0 || w < 0 || ld < w || out->ld < w) return fail(FSG_ERR_INVALID, "bad shape");
  if (out->dtype < FSG_F32 || out->dtype > FSG_I16) return fail(FSG_ERR_DTYPE, "dtype %d", out->dtype);
  if ((long long)h * w == 0) return FSG_OK;
  // scale <= 0 leaves the values unscaled (a no-op normalisation, _global_stats.py:170-171).
  int do_scale = scale > 0.0;
  dim3 b(64, 4);
  dim3 g((w + 63) / 64, (unsigned)std::min((h + 3) / 4, 65535));
  affine_kernel<<<g, b, 0, (cudaStream_t)stream>>>(in_dev, ld, h, w, (float)offset, (float)scale, do_scale,
                                                   clamp_min0, out->ptr, out->ld, out->dtype, out->q_a, out->q_b,
                                                   out->q_min, out->q_max);
  FSG_LAUNCHED(1);
  return FSG_OK;
}
