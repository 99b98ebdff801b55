// topousm_fast's full-resolution box means on the tcgen05 tensor cores.
//
// For the full-resolution radii r (downsample factor 1, 2 <= r <= 32) of a
// tile window, the reference computes uniform_filter(2r+1, 'reflect') means
// (algorithms/_impl_topousm_fast.py:78-87 via handle_nan_with_uniform,
// algorithms/_nan_utils.py:34-47) and accumulates w_r * (z - mean_r).  A box
// sum is two banded Toeplitz products, B_r = V_r Q H_r^T (V_r, H_r: bands of
// ones of width 2r+1), run here as BF16 MMAs with FP32 accumulation in tensor
// memory.  One CTA owns a tile of 128 output rows x 192 output columns of a
// window; its input region is 192 rows x 256 columns ('reflect' at the window
// edges, as scipy).
//
// Arithmetic (windows without NoData; c_r = w_r / (2r+1)^2, W = sum_r w_r):
//   * Fixed point per tile: Q = rint((z - c) 2^k), c the tile's centre
//     elevation, k the largest with |Q| <= 2^22 over the region.
//   * Column offsets: q(i, col) = Q(i, col) - o(col), o(col) = Q(centre row, col).
//     q is split into three BF16 digits (multiples of 2^16, 2^8, 1) whose
//     products with the band of ones are exact.
//   * Pass 1 (vertical, M=128 N=128 K=16 per MMA, two column halves): the high
//     digit accumulates in D1_hi (multiples of 2^16 below 2^30), the two low
//     digits in D1_lo (integers below 2^22): every partial sum is an exact FP32
//     integer, so S1'(y, col) = D1_hi + D1_lo is the exact vertical box sum.
//   * Row offsets: p(y) = S1'(y, centre column).  Pass 2 (horizontal, M=128
//     N=192) accumulates A2 = c_r (S1' - p(y)), split into three BF16 terms
//     (hi + mid + lo, exact), into one FP32 accumulator D2 over all radii.  D2
//     then holds only second differences of the terrain (a plane contributes
//     nothing), which keeps its accumulation error small.
//   * Epilogue: sum_r c_r B_r = D2 + Py(y) + Ox(x), Py = sum_r c_r (2r+1) p_r(y),
//     Ox = sum_r c_r (2r+1) sum_{|col - x| <= r} o(col), and
//     sum_r w_r (z - mean_r) = W (z - c) - 2^-k (D2 + Py + Ox).
// The K dimension runs in reverse (k = K-1-i) on both sides, which makes every
// 8x8 core matrix of a band depend only on the sum of its block indices: each
// band is one compact table of core matrices in shared memory (40 and 56 of
// them) read through descriptors with equal leading and stride offsets.  Only
// the K steps a radius' band reaches are issued.
//
// Roles (416 threads): warps 0-7 stage the digits of q (global -> NoData check
// -> fixed point -> the MN-major B operand of pass 1, a ring of K steps), warp
// 12 allocates tensor memory and one thread issues every MMA, warps 8-11 drain
// D1 into the A operand of pass 2 and run the epilogue (D2 staged through
// shared memory, then per output column the decimated radii, the large-radius
// field, the p99 scale and the int16/uint8 encoding, as the exact kernels do).
// A tile whose input region holds NoData is not written: it goes on a list
// that the exact fixed-point kernel (topousm_hybrid / topousm_fixed) then
// computes, with the NaN-aware means of the reference.
//
// Every wait is bounded; a wait that runs out sets bit 1 of the error word
// (fsg_kernel_errors) and stops the CTA after its tensor memory is freed.
#include <cuda_bf16.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "fsg_topousm.cuh"

namespace fsg {

// Device-side failures of topousm_tc (bit 1: a pipeline wait ran out of polls),
// read and cleared by fsg_kernel_errors through tc_take_errors.
__device__ unsigned g_tc_errors;

// ------------------------------------------------------------------ layout
namespace {

constexpr int TC_TH = 128, TC_TW = 192, TC_HALO = 32;
constexpr int TC_IH = TC_TH + 2 * TC_HALO;  // 192 input rows (pass-1 K)
constexpr int TC_IW = TC_TW + 2 * TC_HALO;  // 256 input columns (pass-2 K)
constexpr int TC_HW = 128;                  // pass-1 column half (MMA N)
constexpr int TC_CROW = 96, TC_CCOL = 128;  // centre row / column of the input region
constexpr int TC_QBITS = 22;                // |Q| <= 2^22
constexpr int TC_NZ = 4, TC_NA = 3;         // ring stages of the two data operands
constexpr int TC_ZSPLIT = 16 * TC_HW * 2;   // one K step of one digit: 16 rows x 128 columns of BF16
constexpr int TC_ZSTAGE = 3 * TC_ZSPLIT;
constexpr int TC_ACOLS = 32;                // one A stage: 32 columns of S1' (two K steps)
constexpr int TC_ASPLIT = TC_TH * TC_ACOLS * 2;
constexpr int TC_ASTAGE = 3 * TC_ASPLIT;
constexpr int TC_T1 = 40 * 128, TC_T2 = 56 * 128, TC_TAB = TC_T1 + TC_T2;  // band tables of one radius
constexpr int TC_PROD = 256;                // producer threads (warps 0-7)
constexpr int TC_EPI0 = 8;                  // first drain / epilogue warp (warps 8-11)
constexpr int TC_MMA_WARP = 12;
constexpr int TC_NT = 13 * 32;
constexpr int TC_EPI_PITCH = 100;           // floats per staged row of 96 outputs
constexpr int TC_D1H_COL = 0, TC_D1L_COL = 128, TC_D2_COL = 256, TC_TMEM_COLS = 512;
constexpr int TC_RT_BYTES = 80;             // per output row: decimated-grid and field row coordinates, Py (hi, lo)
constexpr int TC_PAR_BYTES = 16 + 4 * TC_IW; // per tile: c, 2^-k, k, flags; o(col)

struct TcLayout {
  int nr;
  __host__ __device__ int zring() const { return nr * TC_TAB; }
  __host__ __device__ int aring() const { return zring() + TC_NZ * TC_ZSTAGE; }
  __host__ __device__ int rows() const { return aring() + TC_NA * TC_ASTAGE; }
  __host__ __device__ int params() const { return rows() + TC_TH * TC_RT_BYTES; }
  __host__ __device__ int rowoff() const { return params() + 2 * TC_PAR_BYTES; }  // [192] input-row offsets
  __host__ __device__ int bars() const { return rowoff() + TC_IH * 8; }
  __host__ __device__ int total() const { return bars() + 512; }
};
// barrier block (byte offsets)
constexpr int BZF = 0, BZE = 32, BAF = 64, BAE = 88, BD1F = 112, BD1E = 120, BD2F = 128, BD2E = 136, BTF = 144,
              BFIN = 176, BES = 184, BPS = 192, OTMEM = 200, OABORT = 204, ORED = 256;

// ------------------------------------------------------------- PTX helpers
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void bar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// Bounded wait for the completion of phase `parity`; gives up when another role
// has aborted or after 2^22 polls (then aborts the CTA and flags the error).
__device__ __forceinline__ bool bar_wait(unsigned bar, unsigned parity, volatile unsigned* abort_flag) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    if (done) return true;
    if ((it & 63) == 63 && *abort_flag) return false;
  }
  *abort_flag = 1u;
  atomicOr(&g_tc_errors, 2u);
  return false;
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle: start address, leading (K
// direction) and stride (M/N direction) byte offsets between 8x16-byte core
// matrices, fixed field 0b001 at bits 46-48.
__device__ __forceinline__ uint64_t sdesc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, A/B major
// (0 = K-major, 1 = MN-major), N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, int a_mn, int b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// 32 consecutive 32-bit columns of the warp's 32 TMEM lanes; waits for the load.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  // the wait takes the registers as operands so that no use is scheduled before it
  asm volatile(
      "tcgen05.wait::ld.sync.aligned;"
      : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
        "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]),
        "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]),
        "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
      :
      : "memory");
}
__device__ __forceinline__ void st_shared_v4(unsigned addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

__device__ __forceinline__ uint32_t bf2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t*>(&v); }
// x = hi + mid + lo in BF16 for a pair of FP32 values (exact: each residual of a
// round-to-nearest BF16 split has at most 8 significant bits), packed two per
// word, the first value in the low half (the lower address).
struct Split3 {
  uint32_t h, m, l;
};
__device__ __forceinline__ Split3 split3(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  const float ra = __fsub_rn(a, hf.x), rb = __fsub_rn(b, hf.y);
  const __nv_bfloat162 m = __floats2bfloat162_rn(ra, rb);
  const float2 mf = __bfloat1622float2(m);
  const __nv_bfloat162 l = __floats2bfloat162_rn(__fsub_rn(ra, mf.x), __fsub_rn(rb, mf.y));
  return {bf2_bits(h), bf2_bits(m), bf2_bits(l)};
}
// The three digits of integers |q| <= 2^23 (multiples of 2^16, of 2^8 below
// 2^16 in magnitude, and below 2^8): exact BF16 values, packed as split3.
__device__ __forceinline__ Split3 digits3(int a, int b) {
  const int ha = (a + 0x8000) & ~0xFFFF, hb = (b + 0x8000) & ~0xFFFF;
  const int ra = a - ha, rb = b - hb;
  const int ma = (ra + 0x80) & ~0xFF, mb = (rb + 0x80) & ~0xFF;
  return {bf2_bits(__floats2bfloat162_rn((float)ha, (float)hb)), bf2_bits(__floats2bfloat162_rn((float)ma, (float)mb)),
          bf2_bits(__floats2bfloat162_rn((float)(ra - ma), (float)(rb - mb)))};
}

// Band tables of one radius r (HALO = 32), both in the K-major core-matrix layout
// (8 rows of 16 bytes, element (a, b) at a * 16 + b * 2):
//   pass 1, A = V_r with reversed K:  core s holds 1 where |159 - 8s - a - b| <= r
//   pass 2, B = H_r with reversed K:  core s holds 1 where |223 - 8s - a - b| <= r
__device__ void build_band_tables(unsigned char* tab, int r, int tid, int nt) {
  uint16_t* t1 = reinterpret_cast<uint16_t*>(tab);
  uint16_t* t2 = reinterpret_cast<uint16_t*>(tab + TC_T1);
  const uint16_t one = 0x3F80u;  // BF16 1.0
  for (int e = tid; e < 40 * 64; e += nt) {
    const int s = e >> 6, a = (e >> 3) & 7, b = e & 7;
    t1[e] = abs(159 - 8 * s - a - b) <= r ? one : (uint16_t)0;
  }
  for (int e = tid; e < 56 * 64; e += nt) {
    const int s = e >> 6, a = (e >> 3) & 7, b = e & 7;
    t2[e] = abs(223 - 8 * s - a - b) <= r ? one : (uint16_t)0;
  }
}

}  // namespace

// Launch arguments of topousm_tc (host fills them with tc_prepare / tc_bind).
struct TcArgs {
  const TopoTileK* tiles;
  const int4* items;  // (tile, x0, y0, -): output origin of a CTA tile, window coordinates
  int nitems;
  int nr;
  int radii[TC_MAXNR];
  float cr[TC_MAXNR];                    // w_r / (2r+1)^2
  double crw[TC_MAXNR];                  // c_r (2r+1) = w_r / (2r+1)
  int j1lo[TC_MAXNR], j1hi[TC_MAXNR];    // pass-1 K steps (16 input rows) the band reaches
  int j2lo[TC_MAXNR], j2hi[TC_MAXNR];    // pass-2 K steps (16 input columns)
  int q2lo[TC_MAXNR], q2hi[TC_MAXNR];    // pass-2 A stages (32 columns)
  float wsum;
  StripArgs S;                           // epilogue: field, scale, encoding, output pitch
  StripItem* fix_items;                  // tiles with NoData, for the exact kernel
  int* fix_count;
  unsigned* zmax;                        // max |z| of the staged values (float bits)
};

namespace {

// The A stages of one column half in the order both sides process them: the half
// holding the centre column (input columns 128..255, stages 3..0) first, so that
// its first stage yields p(y); then columns 0..127 (stages 7..4).
__device__ __forceinline__ int stage_lo(const TcArgs& A, int rr, int h) { return max(A.q2lo[rr], h ? 0 : 4); }
__device__ __forceinline__ int stage_hi(const TcArgs& A, int rr, int h) { return min(A.q2hi[rr], h ? 3 : 7); }

__global__ void __launch_bounds__(TC_NT, 1) topousm_tc(const __grid_constant__ TcArgs A) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const TcLayout L{A.nr};
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* bars = sm + L.bars();
  const unsigned sbase = smem_u32(sm);
  const unsigned B = sbase + (unsigned)L.bars();
  volatile unsigned* tmem_slot = reinterpret_cast<volatile unsigned*>(bars + OTMEM);
  volatile unsigned* abort_flag = reinterpret_cast<volatile unsigned*>(bars + OABORT);
  // per tile parameters (two buffers): [0] c, [1] 2^-k, [2] k, [3] NoData flag, then o(col) x 256
  auto params = [&](int titer) { return reinterpret_cast<int*>(sm + L.params() + (titer & 1) * TC_PAR_BYTES); };

  // ---- set-up: band tables, barriers, tensor memory
  for (int r = 0; r < A.nr; ++r) build_band_tables(sm + r * TC_TAB, A.radii[r], tid, TC_NT);
  if (tid == 0) {
    for (int s = 0; s < TC_NZ; ++s) {
      bar_init(B + BZF + 8 * s, TC_PROD);
      bar_init(B + BZE + 8 * s, 1);
    }
    for (int s = 0; s < TC_NA; ++s) {
      bar_init(B + BAF + 8 * s, 128);
      bar_init(B + BAE + 8 * s, 1);
    }
    bar_init(B + BD1F, 1);
    bar_init(B + BD1E, 128);
    bar_init(B + BD2F, 1);
    bar_init(B + BD2E, 128);
    for (int s = 0; s < 4; ++s) bar_init(B + BTF + 8 * s, TC_PROD);
    bar_init(B + BFIN, 1);
    bar_init(B + BES, 128);
    bar_init(B + BPS, TC_PROD);
    *abort_flag = 0u;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == TC_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(B + OTMEM),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();  // band tables: generic writes, read by the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;

  if (warp < TC_PROD / 32) {
    // ================================================ producers: digits of q
    float zmaxv = 0.f;
    unsigned n = 0, psync = 0;
    int titer = 0;
    float* red = reinterpret_cast<float*>(bars + ORED);  // per-warp partial maxima, NoData votes
    // producer-wide barrier on an mbarrier (bounded wait)
    auto prod_sync = [&]() {
      bar_arrive(B + BPS);
      const bool ok = bar_wait(B + BPS, psync & 1u, abort_flag);
      ++psync;
      return ok;
    };
    for (int it = blockIdx.x; it < A.nitems && !*abort_flag; it += gridDim.x, ++titer) {
      const int4 I = A.items[it];
      const ZView z = A.tiles[I.x].z;
      const int x0 = I.y, y0 = I.z;
      const bool nd = z.has_nodata != 0;
      const int xb = x0 - TC_HALO;
      const bool vec = (z.ld & 3) == 0 && ((reinterpret_cast<uintptr_t>(z.p) & 15) == 0) && ((xb & 3) == 0);
      // eight consecutive columns (window column wx0..) of window row wy, 'reflect' at the edges
      auto load8 = [&](int wy, int wx0, float (&v)[8]) {
        const float* row = z.p + (long long)wy * z.ld;
        if (vec && wx0 >= 0 && wx0 + 8 <= z.w) {
          const float4 a4 = __ldg(reinterpret_cast<const float4*>(row + wx0));
          const float4 b4 = __ldg(reinterpret_cast<const float4*>(row + wx0) + 1);
          v[0] = a4.x; v[1] = a4.y; v[2] = a4.z; v[3] = a4.w;
          v[4] = b4.x; v[5] = b4.y; v[6] = b4.z; v[7] = b4.w;
        } else {
#pragma unroll
          for (int e = 0; e < 8; ++e) v[e] = __ldg(row + reflect_idx(wx0 + e, z.w));
        }
      };
      // -- phase A: centre elevation, max |z - c| and NoData over the region, k, o(col)
      float c = __ldg(z.p + (long long)reflect_idx(y0 - TC_HALO + TC_CROW, z.h) * z.ld +
                      reflect_idx(xb + TC_CCOL, z.w));
      if (is_nodata(c, z.ndf, nd)) c = 0.f;
      float mloc = 0.f;
      bool seen = false;
#pragma unroll 4
      for (int item = tid; item < TC_IH * (TC_IW / 8); item += TC_PROD) {
        const int i = item / (TC_IW / 8), g = item - (item / (TC_IW / 8)) * (TC_IW / 8);
        float v[8];
        load8(reflect_idx(y0 - TC_HALO + i, z.h), xb + 8 * g, v);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          if (is_nodata(v[e], z.ndf, nd)) seen = true;
          else {
            mloc = fmaxf(mloc, fabsf(__fsub_rn(v[e], c)));
            zmaxv = fmaxf(zmaxv, fabsf(v[e]));
          }
        }
      }
      for (int o = 16; o > 0; o >>= 1) mloc = fmaxf(mloc, __shfl_xor_sync(0xffffffffu, mloc, o));
      const unsigned anynd = __any_sync(0xffffffffu, seen) ? 1u : 0u;
      if (lane == 0) {
        red[warp] = mloc;
        red[8 + warp] = __uint_as_float(anynd);
      }
      if (!prod_sync()) break;
      float m = 0.f;
      unsigned ndf = 0u;
      for (int w = 0; w < TC_PROD / 32; ++w) {
        m = fmaxf(m, red[w]);
        ndf |= __float_as_uint(red[8 + w]);
      }
      int e2 = 0;
      if (m > 0.f && isfinite(m)) frexpf(m, &e2);   // m < 2^e2
      const int k = max(-60, min(60, TC_QBITS - e2));
      const float sk = ldexpf(1.0f, k);
      int* P = params(titer);
      long long* roff = reinterpret_cast<long long*>(sm + L.rowoff());
      if (tid < TC_IH) roff[tid] = (long long)reflect_idx(y0 - TC_HALO + tid, z.h) * z.ld;  // 'reflect' rows
      {
        // o(col) = Q(centre row, col)
        const float* crow = z.p + (long long)reflect_idx(y0 - TC_HALO + TC_CROW, z.h) * z.ld;
        const float v = __ldg(crow + reflect_idx(xb + tid, z.w));
        P[4 + tid] = is_nodata(v, z.ndf, nd) ? 0 : __float2int_rn(__fmul_rn(__fsub_rn(v, c), sk));
        if (tid == 0) {
          P[0] = __float_as_int(c);
          P[1] = __float_as_int(ldexpf(1.0f, -k));
          P[2] = k;
          P[3] = (int)ndf;
        }
      }
      if (!prod_sync()) break;  // o(col) visible to every producer; red[] free again
      // -- phase B: per radius and column half, the K steps of the band; the next step's
      //    eight values are loaded while this step's are converted and stored
      {
        const int kk = tid & 15, g = tid >> 4;  // row of the K step, 8-column group of the half
        auto fetch = [&](int j, int hh, float (&v)[8]) {
          const int i = TC_IH - 1 - 16 * j - kk;  // reversed K: k = 16 j + kk <-> input row i
          const float* row = z.p + roff[i];
          const int wx0 = xb + TC_HW * hh + 8 * g;
          if (vec && wx0 >= 0 && wx0 + 8 <= z.w) {
            const float4 a4 = __ldg(reinterpret_cast<const float4*>(row + wx0));
            const float4 b4 = __ldg(reinterpret_cast<const float4*>(row + wx0) + 1);
            v[0] = a4.x; v[1] = a4.y; v[2] = a4.z; v[3] = a4.w;
            v[4] = b4.x; v[5] = b4.y; v[6] = b4.z; v[7] = b4.w;
          } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = __ldg(row + reflect_idx(wx0 + e, z.w));
          }
        };
        int rr = 0, hh = 1, j = A.j1lo[0];
        float v[8];
        fetch(j, hh, v);
        bool more = true;
        while (more) {
          int nr = rr, nh = hh, nj = j + 1;  // the step after this one
          if (nj > A.j1hi[nr]) {
            if (nh == 1) {
              nh = 0;
              nj = A.j1lo[nr];
            } else {
              ++nr;
              nh = 1;
              nj = nr < A.nr ? A.j1lo[nr] : 0;
            }
          }
          more = nr < A.nr;
          float vn[8];
          if (more) fetch(nj, nh, vn);
          const int s = (int)(n % TC_NZ);
          const unsigned u = n / TC_NZ;
          if (!bar_wait(B + BZE + 8 * s, (u & 1u) ^ 1u, abort_flag)) goto prod_done;
          const unsigned zs = sbase + (unsigned)(L.zring() + s * TC_ZSTAGE);
          const int col0 = TC_HW * hh + 8 * g;  // input column
          uint32_t hw[4], mw[4], lw[4];
#pragma unroll
          for (int e = 0; e < 8; e += 2) {
            const int qa = is_nodata(v[e], z.ndf, nd) ? 0
                           : __float2int_rn(__fmul_rn(__fsub_rn(v[e], c), sk)) - P[4 + col0 + e];
            const int qb = is_nodata(v[e + 1], z.ndf, nd) ? 0
                           : __float2int_rn(__fmul_rn(__fsub_rn(v[e + 1], c), sk)) - P[4 + col0 + e + 1];
            const Split3 d = digits3(qa, qb);
            hw[e >> 1] = d.h;
            mw[e >> 1] = d.m;
            lw[e >> 1] = d.l;
          }
          // MN-major B operand: element (column n, k) at (n/8)*256 + (k/8)*128 + (k%8)*16 + (n%8)*2
          const unsigned off = (unsigned)(g * 256 + (kk >> 3) * 128 + (kk & 7) * 16);
          st_shared_v4(zs + off, hw[0], hw[1], hw[2], hw[3]);
          st_shared_v4(zs + TC_ZSPLIT + off, mw[0], mw[1], mw[2], mw[3]);
          st_shared_v4(zs + 2 * TC_ZSPLIT + off, lw[0], lw[1], lw[2], lw[3]);
          fence_async_smem();
          bar_arrive(B + BZF + 8 * s);
          ++n;
          rr = nr;
          hh = nh;
          j = nj;
#pragma unroll
          for (int e = 0; e < 8; ++e) v[e] = vn[e];
        }
      }
      bar_arrive(B + BTF + 8 * (titer & 3));
    }
  prod_done:
    for (int o = 16; o > 0; o >>= 1) zmaxv = fmaxf(zmaxv, __shfl_xor_sync(0xffffffffu, zmaxv, o));
    if (lane == 0 && isfinite(zmaxv)) atomicMax(A.zmax, __float_as_uint(zmaxv));
  } else if (warp == TC_MMA_WARP) {
    // ======================================================= MMA issuer
    if (lane == 0) {
      const uint32_t id1 = idesc_bf16(128, TC_HW, 0, 1);  // A = band (K-major), B = digits (MN-major)
      const uint32_t id2 = idesc_bf16(128, TC_TW, 0, 0);  // A = c_r (S1' - p) (K-major), B = band (K-major)
      const unsigned zr = sbase + (unsigned)L.zring(), ar = sbase + (unsigned)L.aring();
      const uint32_t d1h = tmem + TC_D1H_COL, d1l = tmem + TC_D1L_COL, d2 = tmem + TC_D2_COL;
      unsigned n = 0, na = 0, ninst = 0;
      int titer = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < A.nitems && ok; it += gridDim.x, ++titer) {
        bool first2 = true;
        for (int rr = 0; rr < A.nr && ok; ++rr) {
          const unsigned t1 = sbase + (unsigned)(rr * TC_TAB), t2 = t1 + TC_T1;
          for (int hh = 1; hh >= 0 && ok; --hh, ++ninst) {
            // pass 1: D1_hi, D1_lo = V_r q of this column half (D1 must have been drained)
            if (!(ok = bar_wait(B + BD1E, (ninst & 1u) ^ 1u, abort_flag))) break;
            tc_fence_after();
            uint32_t acc = 0;
            for (int j = A.j1lo[rr]; j <= A.j1hi[rr]; ++j, ++n) {
              const int s = (int)(n % TC_NZ);
              if (!(ok = bar_wait(B + BZF + 8 * s, (n / TC_NZ) & 1u, abort_flag))) break;
              tc_fence_after();
              const uint64_t a = sdesc(t1 + (unsigned)(2 * j * 128), 128, 128);
              const unsigned zb = zr + (unsigned)(s * TC_ZSTAGE);
              mma_bf16(d1h, a, sdesc(zb, 128, 256), id1, acc);
              mma_bf16(d1l, a, sdesc(zb + TC_ZSPLIT, 128, 256), id1, acc);
              mma_bf16(d1l, a, sdesc(zb + 2 * TC_ZSPLIT, 128, 256), id1, 1u);
              acc = 1;
              mma_commit(B + BZE + 8 * s);
            }
            if (!ok) break;
            mma_commit(B + BD1F);
            // pass 2: D2 += (c_r (S1' - p)) H_r^T, stage by stage as the drain writes them
            if (first2) {
              if (!(ok = bar_wait(B + BD2E, ((unsigned)titer & 1u) ^ 1u, abort_flag))) break;
              tc_fence_after();
            }
            for (int q = stage_hi(A, rr, hh); q >= stage_lo(A, rr, hh); --q, ++na) {
              const int s = (int)(na % TC_NA);
              if (!(ok = bar_wait(B + BAF + 8 * s, (na / TC_NA) & 1u, abort_flag))) break;
              tc_fence_after();
#pragma unroll
              for (int jl = 0; jl < 2; ++jl) {
                const int j = 2 * q + jl;
                if (j < A.j2lo[rr] || j > A.j2hi[rr]) continue;
                const uint64_t b = sdesc(t2 + (unsigned)(2 * j * 128), 128, 128);
#pragma unroll
                for (int sp = 0; sp < 3; ++sp) {
                  mma_bf16(d2, sdesc(ar + (unsigned)(s * TC_ASTAGE + sp * TC_ASPLIT + jl * 256), 128, 512), b, id2,
                           first2 ? 0u : 1u);
                  first2 = false;
                }
              }
              mma_commit(B + BAE + 8 * s);
            }
          }
        }
        if (ok) mma_commit(B + BD2F);
      }
      // every MMA issued has completed before tensor memory is released
      mma_commit(B + BFIN);
      bar_wait(B + BFIN, 0u, abort_flag);
    }
    __syncwarp();
  } else if (warp >= TC_EPI0 && warp < TC_EPI0 + 4) {
    // ======================================= drain of D1 and the epilogue
    const int m = 32 * (warp & 3) + lane;  // TMEM lane = output row of the tile
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    const int te = tid - TC_EPI0 * 32;     // 0..127
    float* stage = reinterpret_cast<float*>(sm + L.aring());  // D2 staging (the A ring is idle then)
    unsigned char* rtab = sm + L.rows();
    unsigned na = 0, ninst = 0, esync = 0;
    int titer = 0;
    const size_t esz = A.S.dtype == FSG_F32 ? 4 : (A.S.dtype == FSG_I16 ? 2 : 1);
    // Waits are made warp-uniform (the tcgen05.ld that follows them is warp-collective),
    // and the warpgroup synchronises on an mbarrier with a bounded wait, so that a role
    // that gave up cannot leave the others blocked.
    auto wwait = [&](unsigned bar, unsigned parity) {
      const bool ok = bar_wait(bar, parity, abort_flag);
      return __all_sync(0xffffffffu, ok);
    };
    auto epi_sync = [&]() {
      bar_arrive(B + BES);
      const bool ok = bar_wait(B + BES, esync & 1u, abort_flag);
      ++esync;
      return __all_sync(0xffffffffu, ok);
    };
    for (int it = blockIdx.x; it < A.nitems; it += gridDim.x, ++titer) {
      const int4 I = A.items[it];
      bool ok = true;
      double py = 0.0;  // Py(row m) = sum_r c_r (2r+1) p_r(m)
      for (int rr = 0; rr < A.nr && ok; ++rr) {
        const float cr = A.cr[rr];
        int p = 0;
        for (int hh = 1; hh >= 0 && ok; --hh, ++ninst) {
          if (!(ok = wwait(B + BD1F, ninst & 1u))) break;
          tc_fence_after();
          for (int q = stage_hi(A, rr, hh); q >= stage_lo(A, rr, hh); --q, ++na) {
            const int s = (int)(na % TC_NA);
            if (!(ok = wwait(B + BAE + 8 * s, ((na / TC_NA) & 1u) ^ 1u))) break;
            // S1' of input columns c0 .. c0+31, c0 = 224 - 32 q (local column c0 - 128 hh of the half)
            const uint32_t lc = (uint32_t)(TC_IW - TC_ACOLS * (q + 1) - TC_HW * hh);
            uint32_t rh[32], rl[32];
            tmem_ld32(tmem + lane_base + TC_D1H_COL + lc, rh);
            tmem_ld32(tmem + lane_base + TC_D1L_COL + lc, rl);
            int sv[32];
#pragma unroll
            for (int t = 0; t < 32; ++t) sv[t] = __float2int_rn(__uint_as_float(rh[t])) + __float2int_rn(__uint_as_float(rl[t]));
            if (hh == 1 && q == 3) {  // input column 128 = the centre column: p(y)
              p = sv[0];
              py += A.crw[rr] * (double)p;
            }
            float v[32];
#pragma unroll
            for (int t = 0; t < 32; ++t) v[t] = __fmul_rn((float)(sv[t] - p), cr);
            // K-major A operand of pass 2: element (row m, k) at (m%8)*16 + (m/8)*512 + (k/8)*128 + (k%8)*2,
            // local k = 31 - t (reversed columns)
            const unsigned as = sbase + (unsigned)(L.aring() + s * TC_ASTAGE + (m & 7) * 16 + (m >> 3) * 512);
#pragma unroll
            for (int qc = 0; qc < 4; ++qc) {
              uint32_t hw[4], mw[4], lw[4];
#pragma unroll
              for (int w = 0; w < 4; ++w) {
                const Split3 sp = split3(v[31 - 8 * qc - 2 * w], v[30 - 8 * qc - 2 * w]);
                hw[w] = sp.h;
                mw[w] = sp.m;
                lw[w] = sp.l;
              }
              st_shared_v4(as + qc * 128, hw[0], hw[1], hw[2], hw[3]);
              st_shared_v4(as + TC_ASPLIT + qc * 128, mw[0], mw[1], mw[2], mw[3]);
              st_shared_v4(as + 2 * TC_ASPLIT + qc * 128, lw[0], lw[1], lw[2], lw[3]);
            }
            fence_async_smem();
            tc_fence_before();
            bar_arrive(B + BAF + 8 * s);
          }
          if (!ok) break;
          tc_fence_before();
          bar_arrive(B + BD1E);
        }
      }
      if (!ok) break;
      // ---------------------------------------------------------- epilogue
      if (!wwait(B + BD2F, (unsigned)titer & 1u)) break;
      tc_fence_after();
      if (!wwait(B + BTF + 8 * (titer & 3), ((unsigned)titer >> 2) & 1u)) break;
      const int* P = params(titer);
      const float c = __int_as_float(P[0]), isk = __int_as_float(P[1]);
      const bool nanflag = P[3] != 0;
      const TopoTileK& T = A.tiles[I.x];
      const int x0 = I.y, y0 = I.z;
      const int yend = min(y0 + TC_TH, T.cy0 + T.ch), xend = min(x0 + TC_TW, T.cx0 + T.cw);
      if (nanflag) {
        if (te == 0) {
          const int k = atomicAdd(A.fix_count, 1);
          A.fix_items[k] = StripItem{I.x, x0, y0, yend};
        }
        tc_fence_before();
        bar_arrive(B + BD2E);
        continue;
      }
      const ZView z = T.z;
      const StripArgs& S = A.S;
      const bool have_large = S.field != nullptr;
      // row m: decimated-grid and field row coordinates, Py
      {
        int* ri = reinterpret_cast<int*>(rtab + m * TC_RT_BYTES);
        float* rf = reinterpret_cast<float*>(rtab + m * TC_RT_BYTES);
        const int y = y0 + m;
        for (int d = 0; d < T.ndec; ++d) {
          const DecK& Dk = T.dec[d];
          const double cc = (double)y * Dk.zy;
          const int sy = (int)floor(cc);
          ri[3 * d] = clamp_idx(sy, Dk.h);
          ri[3 * d + 1] = clamp_idx(sy + 1, Dk.h);
          rf[3 * d + 2] = (float)(cc - (double)sy);
        }
        if (have_large) {
          const float cy = __fsub_rn(__fmul_rn(__fadd_rn((float)(T.gy0 + y), 0.5f), S.sy), 0.5f);
          const float f0 = floorf(cy);
          ri[12] = clamp_idx((int)f0, S.fh);
          ri[13] = clamp_idx((int)f0 + 1, S.fh);
          rf[14] = cy - f0;
        }
        rf[15] = (float)py;
        rf[16] = (float)(py - (double)rf[15]);  // Py = hi + lo (float-float)
      }
      for (int half = 0; half < 2; ++half) {
#pragma unroll 1
        for (int cs = 0; cs < 3; ++cs) {
          uint32_t v[32];
          tmem_ld32(tmem + lane_base + (uint32_t)(TC_D2_COL + 96 * half + 32 * cs), v);
          float* dst = stage + m * TC_EPI_PITCH + 32 * cs;
#pragma unroll
          for (int t = 0; t < 32; t += 4)
            *reinterpret_cast<float4*>(dst + t) = make_float4(__uint_as_float(v[t]), __uint_as_float(v[t + 1]),
                                                              __uint_as_float(v[t + 2]), __uint_as_float(v[t + 3]));
        }
        if (half == 1) {
          tc_fence_before();
          bar_arrive(B + BD2E);  // D2 may take the next tile's products now
        }
        if (!(ok = epi_sync())) break;
        const int xo = 96 * half + te;  // output column of the tile
        const int x = x0 + xo;
        if (te < 96 && x < xend) {
          // Ox(x) = sum_r c_r (2r+1) sum_{|col - x| <= r} o(col), col = input column
          double ox = 0.0;
          for (int rr = 0; rr < A.nr; ++rr) {
            const int r = A.radii[rr];
            int so = 0;
            for (int col = xo + TC_HALO - r; col <= xo + TC_HALO + r; ++col) so += P[4 + col];
            ox += A.crw[rr] * (double)so;
          }
          const float oxh = (float)ox, oxl = (float)(ox - (double)oxh);  // Ox = hi + lo
          int dxa[ST_MAXD], dxb[ST_MAXD], dya[ST_MAXD];
          float dfx[ST_MAXD], dm[ST_MAXD][4];
#pragma unroll
          for (int d = 0; d < ST_MAXD; ++d) {
            dxa[d] = dxb[d] = 0;
            dya[d] = -1;
            dfx[d] = 0.f;
            dm[d][0] = dm[d][1] = dm[d][2] = dm[d][3] = 0.f;
            if (d < T.ndec) {
              const DecK& Dk = T.dec[d];
              const double cc = (double)x * Dk.zx;
              const int sx = (int)floor(cc);
              dxa[d] = clamp_idx(sx, Dk.w);
              dxb[d] = clamp_idx(sx + 1, Dk.w);
              dfx[d] = (float)(cc - (double)sx);
            }
          }
          int fxa = 0, fxb = 0, fya = INT_MIN;
          float ftx = 0.f, fa = 0.f, fb = 0.f, fc = 0.f, fd = 0.f;
          if (have_large) {
            const float cx = __fsub_rn(__fmul_rn(__fadd_rn((float)(T.gx0 + x), 0.5f), S.sx), 0.5f);
            const float f0 = floorf(cx);
            ftx = cx - f0;
            fxa = clamp_idx((int)f0, S.fw);
            fxb = clamp_idx((int)f0 + 1, S.fw);
          }
          const float* zp = z.p + (long long)y0 * z.ld + x;
          char* op = T.out + ((long long)(y0 - T.cy0) * S.old + (x - T.cx0)) * (long long)esz;
          const long long ostep = S.old * (long long)esz;
          const float wsum = A.wsum;
          for (int mm = 0; mm < yend - y0; ++mm) {
            const float zv = __ldg(zp);
            zp += z.ld;
            const int* ri = reinterpret_cast<const int*>(rtab + mm * TC_RT_BYTES);
            const float* rf = reinterpret_cast<const float*>(rtab + mm * TC_RT_BYTES);
            // sum_r w_r (z - mean_r) = W (z - c) - 2^-k (D2 + Py + Ox)
            // u = D2 + Py + Ox in float-float (Py and Ox are large, D2 second differences only)
            const FF t = two_sum(rf[15], oxh);
            const FF t2 = two_sum(t.hi, stage[mm * TC_EPI_PITCH + te]);
            const float ulo = __fadd_rn(__fadd_rn(t.lo, t2.lo), __fadd_rn(rf[16], oxl));
            // W (z - c) - 2^-k u: the power-of-two scaling is exact and the large terms cancel
            float a = __fsub_rn(__fsub_rn(__fmul_rn(wsum, __fsub_rn(zv, c)), __fmul_rn(t2.hi, isk)), __fmul_rn(ulo, isk));
#pragma unroll
            for (int d = 0; d < ST_MAXD; ++d) {
              if (d >= T.ndec) break;
              const DecK& Dk = T.dec[d];
              const int ya = ri[3 * d];
              if (ya != dya[d]) {
                const int yb = ri[3 * d + 1];
                const float* msd = Dk.ms;
                dm[d][0] = __ldg(msd + (long long)ya * Dk.w + dxa[d]);
                dm[d][1] = __ldg(msd + (long long)ya * Dk.w + dxb[d]);
                dm[d][2] = __ldg(msd + (long long)yb * Dk.w + dxa[d]);
                dm[d][3] = __ldg(msd + (long long)yb * Dk.w + dxb[d]);
                dya[d] = ya;
              }
              const float fy = rf[3 * d + 2], fx = dfx[d];
              const float top = fmaf(fx, dm[d][1] - dm[d][0], dm[d][0]);
              const float bot = fmaf(fx, dm[d][3] - dm[d][2], dm[d][2]);
              const float mean = fmaf(fy, bot - top, top);
              a = __fadd_rn(a, __fmul_rn(Dk.weight, __fsub_rn(zv, mean)));
            }
            float vout = a;
            if (have_large) {
              const int ya = ri[12];
              if (ya != fya) {
                const int yb = ri[13];
                fa = __ldg(S.field + ya * S.fld + fxa);
                fb = __ldg(S.field + ya * S.fld + fxb);
                fc = __ldg(S.field + yb * S.fld + fxa);
                fd = __ldg(S.field + yb * S.fld + fxb);
                fya = ya;
              }
              const float ty = rf[14];
              const float top = fmaf(ftx, fb - fa, fa);
              const float bot = fmaf(ftx, fd - fc, fc);
              vout = __fadd_rn(a, __fsub_rn(__fmul_rn(S.w_large, zv), fmaf(ty, bot - top, top)));
            }
            if (S.scale > 0.f) vout = div_by(vout, S.scale, S.rscale);
            if (S.dtype == FSG_F32) *reinterpret_cast<float*>(op) = vout;
            else if (S.dtype == FSG_U8) *reinterpret_cast<uint8_t*>(op) = (uint8_t)(int)quantize(vout, S.qa, S.qb, S.qmin, S.qmax);
            else *reinterpret_cast<int16_t*>(op) = (int16_t)(int)quantize(vout, S.qa, S.qb, S.qmin, S.qmax);
            op += ostep;
          }
        }
        if (!(ok = epi_sync())) break;  // the staging rows are rewritten by the next half / tile
      }
      if (!ok) break;
    }
  }
  // ---- tear-down: every role is done; release tensor memory
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == TC_MMA_WARP)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

}  // namespace

// ---------------------------------------------------------------------- host
// Pass-1 K steps (reversed input rows) and pass-2 K steps (reversed input
// columns) that radius r's band reaches, for a 128-row, 192-column tile.
static void band_steps(int r, int* j1lo, int* j1hi, int* j2lo, int* j2hi) {
  auto ceil_div = [](int a, int b) { return a >= 0 ? (a + b - 1) / b : -((-a) / b); };
  *j1lo = std::max(0, ceil_div(17 - r, 16));
  *j1hi = std::min(TC_IH / 16 - 1, (159 + r) / 16);
  *j2lo = std::max(0, ceil_div(17 - r, 16));
  *j2hi = std::min(TC_IW / 16 - 1, (223 + r) / 16);
}

int tc_supported(const int* radii, int nfull) {
  if (nfull < 1 || nfull > TC_MAXNR) return 0;
  for (int i = 0; i < nfull; ++i)
    if (radii[i] < 2 || radii[i] > TC_HALO) return 0;
  return 1;
}

int tc_prepare(TcArgs** out, const StripArgs& S, int nfull, size_t* smem) {
  static_assert(sizeof(TcArgs) < 4000, "kernel parameter block");
  TcArgs* A = new TcArgs;
  std::memset(A, 0, sizeof(TcArgs));
  A->nr = nfull;
  A->S = S;
  double wsum = 0.0;
  for (int i = 0; i < nfull; ++i) {
    const int r = S.radii[i];
    A->radii[i] = r;
    A->cr[i] = (float)((double)S.weights[i] / ((double)(2 * r + 1) * (double)(2 * r + 1)));
    A->crw[i] = (double)A->cr[i] * (double)(2 * r + 1);
    // W = sum_r c_r (2r+1)^2 with the same (rounded) c_r, so that a constant offset cancels
    wsum += (double)A->cr[i] * (double)(2 * r + 1) * (double)(2 * r + 1);
    band_steps(r, &A->j1lo[i], &A->j1hi[i], &A->j2lo[i], &A->j2hi[i]);
    A->q2lo[i] = A->j2lo[i] / 2;
    A->q2hi[i] = A->j2hi[i] / 2;
    // the drain takes p(y) from stage 3 (input column 128), the first it processes
    if (A->q2lo[i] > 3 || A->q2hi[i] < 3) {
      delete A;
      return fail(FSG_ERR_UNSUPPORTED, "tensor topousm: radius %d", r);
    }
  }
  A->wsum = (float)wsum;
  *smem = (size_t)TcLayout{nfull}.total();
  FSG_CUDA(cudaFuncSetAttribute(topousm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem));
  *out = A;
  return FSG_OK;
}

void tc_release(TcArgs* A) { delete A; }

void tc_bind(TcArgs* A, const TopoTileK* tiles, const int4* items, int nitems, StripItem* fix_items, int* fix_count,
             unsigned* zmax) {
  A->tiles = tiles;
  A->items = items;
  A->nitems = nitems;
  A->fix_items = fix_items;
  A->fix_count = fix_count;
  A->zmax = zmax;
}

int tc_take_errors(unsigned* flags) {
  unsigned v = 0;
  FSG_CUDA(cudaMemcpyFromSymbol(&v, g_tc_errors, sizeof(v)));
  const unsigned zero = 0;
  FSG_CUDA(cudaMemcpyToSymbol(g_tc_errors, &zero, sizeof(zero)));
  *flags = v;
  return FSG_OK;
}

void tc_items(const TopoTileK* tk, int ntiles, std::vector<int4>* items) {
  for (int t = 0; t < ntiles; ++t) {
    const TopoTileK& T = tk[t];
    if (T.ch <= 0 || T.cw <= 0) continue;
    for (int y = T.cy0; y < T.cy0 + T.ch; y += TC_TH)
      for (int x = T.cx0; x < T.cx0 + T.cw; x += TC_TW) items->push_back(make_int4(t, x, y, 0));
  }
}

int tc_launch(const TcArgs* A, size_t smem, cudaStream_t s) {
  if (A->nitems <= 0) return FSG_OK;
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  const int grid = std::min(A->nitems, di.sms);
  topousm_tc<<<grid, TC_NT, smem, s>>>(*A);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

}  // namespace fsg
