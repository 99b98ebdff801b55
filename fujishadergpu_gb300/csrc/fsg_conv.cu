// Convolution kernels of the openness surrogate: 3x3 dilated convolutions of
// 32-channel feature maps as implicit GEMMs on the tensor cores
// (mma.sync m16n8k16, BF16 operands, FP32 accumulation), their data and
// weight gradients, and the 1x1 output head.
//
// Feature maps are float32 [B][H][W][C] with the channel fastest (C = 32, or 16
// for the zero-padded 3-channel input), W a multiple of 16.  A warp owns 16
// consecutive pixels of a row and all 32 output channels: per tap and
// 16-channel slice one A fragment (16 pixels x 16 channels, converted to BF16
// on the fly, zero outside the map) against four B fragments (16 channels x 8
// output channels) from the BF16 weight table in shared memory.
//   forward     y = act(sum_tap x(p + tap*dil) W[tap] + b) (+ r)
//   data grad   the same kernel with the taps mirrored and W transposed
//   weight grad dW[tap] += X(p + tap*dil)^T G(p): M = 32 input channels,
//               N = 32 output channels, K = pixels, atomically reduced
#include <algorithm>
#include <cstring>
#include <vector>

#include "fsg_common.cuh"

namespace fsg {
namespace {

constexpr int CO = 32;       // output channels of every 3x3 layer
constexpr int CW_NT = 256;   // threads per block (8 warps)

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  unsigned r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

__device__ __forceinline__ void mma_bf16(float* d, const unsigned* a, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float2 ld2(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }

struct ConvArgs {
  const float* x;       // [B][H][W][CIN]
  float* y;             // [B][H][W][32]
  const float* res;     // nullable, added after the activation
  const float* bias;    // nullable [32]
  const unsigned* wb;   // BF16 pairs [9][CIN/16][32 (n)][8 (k pairs)]
  int B, H, W, dil;
  int relu;
  int flip;             // mirrored taps (data gradient)
};

template <int CIN>
__global__ void __launch_bounds__(CW_NT) conv3x3_mma(const __grid_constant__ ConvArgs A) {
  constexpr int KC = CIN / 16;
  __shared__ unsigned ws[9 * KC * CO * 8];
  for (int i = threadIdx.x; i < 9 * KC * CO * 8; i += CW_NT) ws[i] = A.wb[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int wpb = CW_NT / 32;
  const long long hw = (long long)A.H * A.W;
  const long long runs = (long long)A.B * hw / 16;
  for (long long run = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); run < runs; run += (long long)gridDim.x * wpb) {
    const long long p0 = run * 16;
    const int bi = (int)(p0 / hw);
    const long long rem = p0 - (long long)bi * hw;
    const int y = (int)(rem / A.W), x0 = (int)(rem - (long long)y * A.W);
    float acc[4][4];
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[n][e] = 0.f;
#pragma unroll 1
    for (int tap = 0; tap < 9; ++tap) {
      int dy = (tap / 3 - 1) * A.dil, dx = (tap % 3 - 1) * A.dil;
      if (A.flip) {
        dy = -dy;
        dx = -dx;
      }
      const int yy = y + dy, xa = x0 + g + dx, xb = xa + 8;
      const bool rok = yy >= 0 && yy < A.H;
      const bool oka = rok && xa >= 0 && xa < A.W, okb = rok && xb >= 0 && xb < A.W;
      const float* pa = A.x + (((long long)bi * A.H + yy) * A.W + xa) * CIN + 2 * t;
      const float* pb = pa + 8 * CIN;
#pragma unroll
      for (int kc = 0; kc < KC; ++kc) {
        const float2 z2 = make_float2(0.f, 0.f);
        const float2 a0 = oka ? ld2(pa + kc * 16) : z2, a2 = oka ? ld2(pa + kc * 16 + 8) : z2;
        const float2 a1 = okb ? ld2(pb + kc * 16) : z2, a3 = okb ? ld2(pb + kc * 16 + 8) : z2;
        const unsigned af[4] = {pack_bf16(a0.x, a0.y), pack_bf16(a1.x, a1.y), pack_bf16(a2.x, a2.y),
                                pack_bf16(a3.x, a3.y)};
        const unsigned* wt = ws + ((tap * KC + kc) * CO + g) * 8 + t;
#pragma unroll
        for (int n = 0; n < 4; ++n) mma_bf16(acc[n], af, wt[n * 64], wt[n * 64 + 4]);
      }
    }
    // epilogue: acc[n][0..1] -> pixel x0+g, channels 8n+2t, +1; acc[n][2..3] -> pixel x0+g+8
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long pix = p0 + g + 8 * h;
      float* yp = A.y + pix * CO;
      const float* rp = A.res ? A.res + pix * CO : nullptr;
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const int c = 8 * n + 2 * t;
        float v0 = acc[n][2 * h], v1 = acc[n][2 * h + 1];
        if (A.bias) {
          v0 += A.bias[c];
          v1 += A.bias[c + 1];
        }
        if (A.relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (rp) {
          const float2 r = ld2(rp + c);
          v0 += r.x;
          v1 += r.y;
        }
        *reinterpret_cast<float2*>(yp + c) = make_float2(v0, v1);
      }
    }
  }
}

// BF16 weight table from float32 weights w[9][cin][32]; transpose: the table of
// the data gradient (input channels <-> output channels, requires cin == 32).
__global__ void pack_weights(const float* w, int cin, int cin_pad, int transpose, unsigned* wb) {
  const int KC = cin_pad / 16;
  const int n_items = 9 * KC * CO * 8;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_items; i += gridDim.x * blockDim.x) {
    const int j = i & 7, n = (i >> 3) & (CO - 1), kc = (i >> 8) % KC, tap = (i >> 8) / KC;
    const int k0 = kc * 16 + 2 * j, k1 = k0 + 1;
    float v0 = 0.f, v1 = 0.f;
    if (!transpose) {
      if (k0 < cin) v0 = w[(tap * cin + k0) * CO + n];
      if (k1 < cin) v1 = w[(tap * cin + k1) * CO + n];
    } else {  // table entry (k = output channel of the forward conv, n = its input channel)
      v0 = w[(tap * cin + n) * CO + k0];
      v1 = w[(tap * cin + n) * CO + k1];
    }
    wb[i] = pack_bf16(v0, v1);
  }
}

struct WgradArgs {
  const float* x;   // [B][H][W][CIN] layer input
  const float* gz;  // [B][H][W][32] gradient at the pre-activation
  float* dw;        // [9][CIN][32] accumulated (atomics)
  int B, H, W, dil, cin;
  long long px_per_warp;
};

// dW[tap][ci][co] += sum_p x(p + tap*dil)[ci] * gz(p)[co]; A = x^T (rows ci),
// B = gz (cols co), K = 16 pixels per MMA step.
template <int CIN>
__global__ void __launch_bounds__(CW_NT) conv3x3_wgrad_mma(const __grid_constant__ WgradArgs A) {
  constexpr int MT = CIN / 16;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long long hw = (long long)A.H * A.W;
  const long long npix = (long long)A.B * hw;
  const long long warp = (long long)blockIdx.x * (CW_NT / 32) + (threadIdx.x >> 5);
  const long long pbeg = warp * A.px_per_warp;
  if (pbeg >= npix) return;
  const long long pend = min(npix, pbeg + A.px_per_warp);
#pragma unroll 1
  for (int tap = 0; tap < 9; ++tap) {
    const int dy = (tap / 3 - 1) * A.dil, dx = (tap % 3 - 1) * A.dil;
    float acc[MT][4][4];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[m][n][e] = 0.f;
    for (long long p0 = pbeg; p0 < pend; p0 += 16) {
      // the four pixels of this lane in the K slice: p0 + 2t, +1, +8, +9
      float xv[4][MT][2];  // [pixel][m tile][row g / g+8]
      float gv[4][4];      // [pixel][n tile]
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const long long p = p0 + 2 * t + (q & 1) + 8 * (q >> 1);
        bool in = p < pend;
        const int bi = (int)(p / hw);
        const long long rem = p - (long long)bi * hw;
        const int y = (int)(rem / A.W), x = (int)(rem - (long long)y * A.W);
        const int ys = y + dy, xs = x + dx;
        const bool ok = in && ys >= 0 && ys < A.H && xs >= 0 && xs < A.W;
        const float* xp = A.x + (((long long)bi * A.H + ys) * A.W + xs) * CIN;
        const float* gp = A.gz + p * CO;
#pragma unroll
        for (int m = 0; m < MT; ++m) {
          xv[q][m][0] = ok ? __ldg(xp + 16 * m + g) : 0.f;
          xv[q][m][1] = ok ? __ldg(xp + 16 * m + g + 8) : 0.f;
        }
#pragma unroll
        for (int n = 0; n < 4; ++n) gv[q][n] = in ? __ldg(gp + 8 * n + g) : 0.f;
      }
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        // A (16 ci x 16 px): a0 (row g, k 2t..2t+1), a1 (row g+8), a2 (row g, k+8), a3 (row g+8, k+8)
        const unsigned af[4] = {pack_bf16(xv[0][m][0], xv[1][m][0]), pack_bf16(xv[0][m][1], xv[1][m][1]),
                                pack_bf16(xv[2][m][0], xv[3][m][0]), pack_bf16(xv[2][m][1], xv[3][m][1])};
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          // B (16 px x 8 co): b0 (k 2t..2t+1, col g), b1 (k 2t+8..2t+9, col g)
          mma_bf16(acc[m][n], af, pack_bf16(gv[0][n], gv[1][n]), pack_bf16(gv[2][n], gv[3][n]));
        }
      }
    }
    // acc[m][n]: rows ci = 16m + g (+8), cols co = 8n + 2t (+1)
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int ci = 16 * m + g + 8 * (e >> 1), co = 8 * n + 2 * t + (e & 1);
          if (ci < A.cin) atomicAdd(A.dw + ((long long)tap * A.cin + ci) * CO + co, acc[m][n][e]);
        }
  }
}

// 1x1 head: out[p] = sum_c h[p][c] w[c] + b (float32).
__global__ void head_fwd(const float* h, const float* w, float b, long long n, float* out) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float* hp = h + p * CO;
    float s = b;
#pragma unroll
    for (int c = 0; c < CO; c += 4) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(hp + c));
      s = fmaf(v.x, w[c], s);
      s = fmaf(v.y, w[c + 1], s);
      s = fmaf(v.z, w[c + 2], s);
      s = fmaf(v.w, w[c + 3], s);
    }
    out[p] = s;
  }
}

// Head gradients: gh[p][c] = go[p] w[c] (+ gres[p][c]); gw[c] += sum_p h[p][c] go[p]; gb += sum_p go[p].
__global__ void head_bwd(const float* h, const float* w, const float* go, const float* gres, long long n, float* gh,
                         float* gw, float* gb) {
  float sw[CO];
#pragma unroll
  for (int c = 0; c < CO; ++c) sw[c] = 0.f;
  float sb = 0.f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float g = go[p];
    sb += g;
#pragma unroll
    for (int c = 0; c < CO; ++c) {
      sw[c] = fmaf(h[p * CO + c], g, sw[c]);
      gh[p * CO + c] = fmaf(g, w[c], gres ? gres[p * CO + c] : 0.f);
    }
  }
#pragma unroll
  for (int c = 0; c < CO; ++c) {
    float v = sw[c];
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(gw + c, v);
  }
  for (int o = 16; o; o >>= 1) sb += __shfl_down_sync(0xffffffffu, sb, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(gb, sb);
}

}  // namespace
}  // namespace fsg

using namespace fsg;

static int conv_grid(long long work, int per_block) {
  DeviceInfo di;
  if (device_info(&di)) return 1;
  const long long blocks = (work + per_block - 1) / per_block;
  return (int)std::max<long long>(1, std::min<long long>(blocks, (long long)di.sms * 16));
}

extern "C" int fsg_conv_pack_weights(const float* w_dev, int32_t cin, int32_t transpose, uint32_t* wb_dev,
                                     void* stream) {
  if (!w_dev || !wb_dev) return fail(FSG_ERR_INVALID, "null array");
  if (cin < 1 || cin > 32 || (transpose && cin != 32)) return fail(FSG_ERR_INVALID, "cin %d", cin);
  const int cin_pad = cin <= 16 ? 16 : 32;
  pack_weights<<<16, 256, 0, (cudaStream_t)stream>>>(w_dev, cin, cin_pad, transpose, reinterpret_cast<unsigned*>(wb_dev));
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_conv3x3(const float* x_dev, int32_t cin_pad, int32_t batch, int32_t h, int32_t w, int32_t dil,
                           const uint32_t* wb_dev, const float* bias_dev, int32_t relu, int32_t flip,
                           const float* res_dev, float* y_dev, void* stream) {
  if (!x_dev || !wb_dev || !y_dev) return fail(FSG_ERR_INVALID, "null array");
  if (cin_pad != 16 && cin_pad != 32) return fail(FSG_ERR_INVALID, "cin_pad %d (16 or 32)", cin_pad);
  if (batch < 1 || h < 1 || w < 16 || (w % 16) != 0 || dil < 1)
    return fail(FSG_ERR_SHAPE, "feature map %d x %d x %d (width a multiple of 16), dilation %d", batch, h, w, dil);
  ConvArgs A;
  A.x = x_dev;
  A.y = y_dev;
  A.res = res_dev;
  A.bias = bias_dev;
  A.wb = wb_dev;
  A.B = batch;
  A.H = h;
  A.W = w;
  A.dil = dil;
  A.relu = relu;
  A.flip = flip;
  const long long runs = (long long)batch * h * w / 16;
  const int grid = conv_grid(runs, CW_NT / 32);
  if (cin_pad == 16) conv3x3_mma<16><<<grid, CW_NT, 0, (cudaStream_t)stream>>>(A);
  else conv3x3_mma<32><<<grid, CW_NT, 0, (cudaStream_t)stream>>>(A);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_conv3x3_wgrad(const float* x_dev, int32_t cin, int32_t cin_pad, int32_t batch, int32_t h,
                                 int32_t w, int32_t dil, const float* gz_dev, float* dw_dev, void* stream) {
  if (!x_dev || !gz_dev || !dw_dev) return fail(FSG_ERR_INVALID, "null array");
  if ((cin_pad != 16 && cin_pad != 32) || cin < 1 || cin > cin_pad) return fail(FSG_ERR_INVALID, "cin %d/%d", cin, cin_pad);
  if (batch < 1 || h < 1 || w < 1 || dil < 1) return fail(FSG_ERR_SHAPE, "bad feature map");
  WgradArgs A;
  A.x = x_dev;
  A.gz = gz_dev;
  A.dw = dw_dev;
  A.B = batch;
  A.H = h;
  A.W = w;
  A.dil = dil;
  A.cin = cin;
  const long long npix = (long long)batch * h * w;
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  const long long warps = std::max<long long>(1, std::min<long long>((npix + 255) / 256, (long long)di.sms * 16));
  A.px_per_warp = ((npix + warps - 1) / warps + 15) / 16 * 16;
  const long long nwarps = (npix + A.px_per_warp - 1) / A.px_per_warp;
  const int grid = (int)((nwarps + CW_NT / 32 - 1) / (CW_NT / 32));
  if (cin_pad == 16) conv3x3_wgrad_mma<16><<<grid, CW_NT, 0, (cudaStream_t)stream>>>(A);
  else conv3x3_wgrad_mma<32><<<grid, CW_NT, 0, (cudaStream_t)stream>>>(A);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_head_forward(const float* h_dev, const float* w_dev, float bias, int64_t npix, float* out_dev,
                                void* stream) {
  if (!h_dev || !w_dev || !out_dev) return fail(FSG_ERR_INVALID, "null array");
  if (npix <= 0) return FSG_OK;
  head_fwd<<<conv_grid(npix, 256), 256, 0, (cudaStream_t)stream>>>(h_dev, w_dev, bias, npix, out_dev);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

extern "C" int fsg_head_backward(const float* h_dev, const float* w_dev, const float* gout_dev, const float* gres_dev,
                                 int64_t npix, float* gh_dev, float* gw_dev, float* gb_dev, void* stream) {
  if (!h_dev || !w_dev || !gout_dev || !gh_dev || !gw_dev || !gb_dev) return fail(FSG_ERR_INVALID, "null array");
  if (npix <= 0) return FSG_OK;
  head_bwd<<<conv_grid(npix, 256), 256, 0, (cudaStream_t)stream>>>(h_dev, w_dev, gout_dev, gres_dev, npix, gh_dev,
                                                                  gw_dev, gb_dev);
  FSG_LAUNCHED(1);
  return FSG_OK;
}
