// Exact order statistics of float32 data (NaN excluded) for the global
// normalisation stats: p99(|x|) of topousm_fast (_normalization.py:21-32) and
// (p1, p99) of openness (_global_stats.py:181-203).
//
// Each requested rank is found by a three-pass radix select (11 + 11 + 10
// bits) over the order-preserving uint32 image of the float32 values; the
// per-pass bin choice runs on the device, so a percentile costs 1 + 3 * ranks
// streaming passes and a single host synchronisation.  The linear
// interpolation between neighbouring ranks follows numpy.percentile's
// 'linear' method (virtual index (n - 1) * q, _lerp), evaluated in FP64
// (NumPy and CuPy interpolate float32 data in float32 for a scalar q; the two
// differ by at most one float32 ulp of the result).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "fsg_common.cuh"

namespace fsg {
namespace {

constexpr int NT = 256;
constexpr int BINS = 2048;

__device__ __forceinline__ unsigned ordered_key(float v) {
  unsigned u = __float_as_uint(v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float key_to_float(unsigned k) {
  unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

struct SelState {
  unsigned prefix;       // selected high bits so far
  unsigned mask;         // which bits of prefix are fixed
  unsigned long long k;  // rank still to find within the current bucket
  unsigned long long hist[BINS];
};

__device__ __forceinline__ bool take(float v, int absmode, unsigned* key) {
  if (v != v) return false;
  if (absmode) v = fabsf(v);
  *key = ordered_key(v);
  return true;
}

__global__ void count_valid(const float* __restrict__ x, long long n, int absmode, unsigned long long* out) {
  unsigned long long c = 0;
  for (long long i = blockIdx.x * (long long)NT + threadIdx.x; i < n; i += (long long)gridDim.x * NT) {
    unsigned k;
    c += take(__ldg(x + i), absmode, &k);
  }
  for (int o = 16; o; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, c);
}

__global__ void hist_pass(const float* __restrict__ x, long long n, int absmode, SelState* st, int shift,
                          int bits) {
  __shared__ unsigned h[BINS];
  for (int i = threadIdx.x; i < BINS; i += NT) h[i] = 0;
  __syncthreads();
  const unsigned prefix = st->prefix, mask = st->mask;
  const unsigned bm = (1u << bits) - 1u;
  for (long long i = blockIdx.x * (long long)NT + threadIdx.x; i < n; i += (long long)gridDim.x * NT) {
    unsigned k;
    if (take(__ldg(x + i), absmode, &k) && (k & mask) == prefix) atomicAdd(&h[(k >> shift) & bm], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < BINS; i += NT)
    if (h[i]) atomicAdd(&st->hist[i], (unsigned long long)h[i]);
}

// Picks the bin holding rank k, narrows the prefix and clears the histogram.
__global__ void pick_bin(SelState* st, int shift, int bits) {
  if (threadIdx.x != 0) return;
  unsigned long long k = st->k;
  int nb = 1 << bits;
  int b = 0;
  for (; b < nb; ++b) {
    unsigned long long c = st->hist[b];
    if (k < c) break;
    k -= c;
  }
  if (b == nb) b = nb - 1;  // unreachable for a valid rank
  st->k = k;
  st->prefix |= (unsigned)b << shift;
  st->mask |= ((1u << bits) - 1u) << shift;
  for (int i = 0; i < BINS; ++i) st->hist[i] = 0;
}

__global__ void init_state(SelState* st, unsigned long long k) {
  st->prefix = 0;
  st->mask = 0;
  st->k = k;
  for (int i = 0; i < BINS; ++i) st->hist[i] = 0;
}

}  // namespace

// Selects the k-th smallest valid value (0-based) into *out_key (device).
static int select_rank(const float* x, long long n, int absmode, unsigned long long k, SelState* st, int grid,
                       cudaStream_t s) {
  init_state<<<1, 1, 0, s>>>(st, k);
  FSG_LAUNCHED(1);
  const int shifts[3] = {21, 10, 0};
  const int bits[3] = {11, 11, 10};
  for (int p = 0; p < 3; ++p) {
    hist_pass<<<grid, NT, 0, s>>>(x, n, absmode, st, shifts[p], bits[p]);
    FSG_LAUNCHED(1);
    pick_bin<<<1, 32, 0, s>>>(st, shifts[p], bits[p]);
    FSG_LAUNCHED(1);
  }
  return FSG_OK;
}

// numpy.percentile(method='linear') index arithmetic (numpy/lib/_function_base_impl.py
// _compute_virtual_index / _get_indexes / _lerp), for one q in [0, 100].
struct LinearPick {
  long long lo, hi;
  double gamma;
};
static LinearPick linear_pick(long long n, double q) {
  double qq = q / 100.0;
  double virt = (double)(n - 1) * qq;  // the 'linear' method's virtual index
  LinearPick p;
  double prev = std::floor(virt);
  p.gamma = virt - prev;
  p.lo = (long long)prev;
  p.hi = p.lo + 1;
  if (virt >= (double)(n - 1)) {
    p.lo = p.hi = n - 1;
  } else if (virt < 0.0) {
    p.lo = p.hi = 0;
  }
  return p;
}

// numpy's _lerp in FP64: a + (b - a) t, or b - (b - a)(1 - t) for t >= 0.5.
static double lerp_numpy(float a, float b, double t) {
  double diff = (double)b - (double)a;
  double r = (double)a + diff * t;
  if (t >= 0.5) r = (double)b - diff * (1.0 - t);
  return r;
}

}  // namespace fsg

using namespace fsg;

extern "C" int fsg_percentile(const float* values_dev, int64_t n, int32_t abs_values, const double* q, int32_t nq,
                              double* out, int64_t* nvalid, void* stream) {
  if ((n > 0 && !values_dev) || nq < 0 || (nq > 0 && (!q || !out))) return fail(FSG_ERR_INVALID, "null argument");
  for (int i = 0; i < nq; ++i)
    if (!(q[i] >= 0.0 && q[i] <= 100.0)) return fail(FSG_ERR_INVALID, "percentile %g outside [0, 100]", q[i]);
  cudaStream_t s = (cudaStream_t)stream;
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  StreamScratch scratch;
  st = scratch.alloc(sizeof(SelState) + 64, s);
  if (st) return st;
  SelState* state = static_cast<SelState*>(scratch.ptr);
  unsigned long long* cnt_dev = reinterpret_cast<unsigned long long*>(static_cast<char*>(scratch.ptr) +
                                                                      sizeof(SelState));
  int grid = (int)std::max<long long>(1, std::min<long long>((n + NT - 1) / NT, (long long)di.sms * 8));
  FSG_CUDA(cudaMemsetAsync(cnt_dev, 0, sizeof(unsigned long long), s));
  if (n > 0) {
    count_valid<<<grid, NT, 0, s>>>(values_dev, n, abs_values, cnt_dev);
    FSG_LAUNCHED(1);
  }
  unsigned long long nv = 0;
  FSG_CUDA(cudaMemcpyAsync(&nv, cnt_dev, sizeof(nv), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  if (nvalid) *nvalid = (int64_t)nv;
  if (nv == 0) {
    for (int i = 0; i < nq; ++i) out[i] = std::nan("");
    return FSG_OK;
  }
  // distinct ranks needed
  std::vector<unsigned long long> ranks;
  std::vector<LinearPick> picks(nq);
  for (int i = 0; i < nq; ++i) {
    picks[i] = linear_pick((long long)nv, q[i]);
    ranks.push_back((unsigned long long)picks[i].lo);
    ranks.push_back((unsigned long long)picks[i].hi);
  }
  std::sort(ranks.begin(), ranks.end());
  ranks.erase(std::unique(ranks.begin(), ranks.end()), ranks.end());
  std::vector<unsigned> keys(ranks.size());
  StreamScratch keys_dev;
  st = keys_dev.alloc(sizeof(unsigned) * ranks.size(), s);
  if (st) return st;
  for (size_t r = 0; r < ranks.size(); ++r) {
    st = select_rank(values_dev, n, abs_values, ranks[r], state, grid, s);
    if (st) return st;
    FSG_CUDA(cudaMemcpyAsync(static_cast<unsigned*>(keys_dev.ptr) + r, &state->prefix, sizeof(unsigned),
                             cudaMemcpyDeviceToDevice, s));
  }
  FSG_CUDA(cudaMemcpyAsync(keys.data(), keys_dev.ptr, sizeof(unsigned) * keys.size(), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  auto value_of = [&](unsigned long long rank) {
    size_t i = std::lower_bound(ranks.begin(), ranks.end(), rank) - ranks.begin();
    return key_to_float(keys[i]);
  };
  for (int i = 0; i < nq; ++i) {
    float a = value_of((unsigned long long)picks[i].lo), b = value_of((unsigned long long)picks[i].hi);
    out[i] = lerp_numpy(a, b, picks[i].gamma);
  }
  return FSG_OK;
}

namespace fsg {
namespace {
// hist[(key >> shift) & (2^bits - 1)] += 1 for the valid keys with (key & mask) == prefix.
__global__ void key_hist(const float* __restrict__ x, long long n, int absmode, unsigned prefix, unsigned mask,
                         int shift, int bits, unsigned long long* hist) {
  __shared__ unsigned h[BINS];
  for (int i = threadIdx.x; i < BINS; i += NT) h[i] = 0;
  __syncthreads();
  const unsigned bm = (1u << bits) - 1u;
  for (long long i = blockIdx.x * (long long)NT + threadIdx.x; i < n; i += (long long)gridDim.x * NT) {
    unsigned k;
    if (take(__ldg(x + i), absmode, &k) && (k & mask) == prefix) atomicAdd(&h[(k >> shift) & bm], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= (int)bm; i += NT)
    if (h[i]) atomicAdd(&hist[i], (unsigned long long)h[i]);
}
}  // namespace
}  // namespace fsg

extern "C" int fsg_key_histogram(const float* values_dev, int64_t n, int32_t abs_values, uint32_t prefix,
                                 uint32_t mask, int32_t shift, int32_t bits, uint64_t* hist_out, void* stream) {
  if ((n > 0 && !values_dev) || !hist_out) return fail(FSG_ERR_INVALID, "null argument");
  if (bits < 1 || bits > 11 || shift < 0 || shift + bits > 32)
    return fail(FSG_ERR_INVALID, "bits %d / shift %d outside the 11-bit radix passes", bits, shift);
  cudaStream_t s = (cudaStream_t)stream;
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  const size_t nb = (size_t)1 << bits;
  StreamScratch scratch;
  st = scratch.alloc(nb * sizeof(unsigned long long), s);
  if (st) return st;
  unsigned long long* h = static_cast<unsigned long long*>(scratch.ptr);
  FSG_CUDA(cudaMemsetAsync(h, 0, nb * sizeof(unsigned long long), s));
  if (n > 0) {
    const int grid = (int)std::max<long long>(1, std::min<long long>((n + NT - 1) / NT, (long long)di.sms * 8));
    key_hist<<<grid, NT, 0, s>>>(values_dev, n, abs_values, prefix, mask, shift, bits, h);
    FSG_LAUNCHED(1);
  }
  FSG_CUDA(cudaMemcpyAsync(hist_out, h, nb * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  return FSG_OK;
}

namespace fsg {
namespace {
__global__ void moments_kernel(const float* __restrict__ x, long long n, double centre, double* acc) {
  // acc[0] += sum(v - centre), acc[1] += sum((v - centre)^2), acc[2] += count (valid v)
  double s = 0.0, s2 = 0.0;
  unsigned long long c = 0;
  for (long long i = blockIdx.x * (long long)NT + threadIdx.x; i < n; i += (long long)gridDim.x * NT) {
    float v = __ldg(x + i);
    if (v == v) {
      double d = (double)v - centre;
      s += d;
      s2 += d * d;
      ++c;
    }
  }
  for (int o = 16; o; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(acc, s);
    atomicAdd(acc + 1, s2);
    atomicAdd(reinterpret_cast<unsigned long long*>(acc + 2), c);
  }
}
}  // namespace
}  // namespace fsg

// Population standard deviation (ddof 0) of the valid values: two FP64 passes
// (mean, then the centred sum of squares).
extern "C" int fsg_std(const float* values_dev, int64_t n, double* out, void* stream) {
  if ((n > 0 && !values_dev) || !out) return fail(FSG_ERR_INVALID, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  StreamScratch scratch;
  st = scratch.alloc(3 * sizeof(double), s);
  if (st) return st;
  int grid = (int)std::max<long long>(1, std::min<long long>((n + NT - 1) / NT, (long long)di.sms * 8));
  double h[3];
  double centre = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    FSG_CUDA(cudaMemsetAsync(scratch.ptr, 0, 3 * sizeof(double), s));
    if (n > 0) {
      moments_kernel<<<grid, NT, 0, s>>>(values_dev, n, centre, static_cast<double*>(scratch.ptr));
      FSG_LAUNCHED(1);
    }
    FSG_CUDA(cudaMemcpyAsync(h, scratch.ptr, sizeof(h), cudaMemcpyDeviceToHost, s));
    FSG_CUDA(cudaStreamSynchronize(s));
    unsigned long long c;
    memcpy(&c, &h[2], 8);
    if (c == 0) {
      *out = std::nan("");
      return FSG_OK;
    }
    if (pass == 0) centre = h[0] / (double)c;
    else *out = std::sqrt(h[1] / (double)c);
  }
  return FSG_OK;
}

// ---------------------------------------------------------------------------
// Percentiles without any allocation.
//
// Some callers cannot allocate device memory during a run: a host application
// whose GPU memory is owned and budgeted by its own pool (every byte must come
// from that pool), or a latency-critical caller that cannot accept the
// implicit device synchronisation cudaMalloc / cudaFree may cause.  For them
// fsg_percentile_noalloc keeps its scratch (the radix-select state, the valid
// count and the selected keys) in the fixed array below, which every GPU that
// loads this library holds until the process exits.
namespace fsg {
namespace {

constexpr int kNoAllocMaxQ = 16;  // at most 16 percentiles per call (32 ranks)
struct NoAllocScratch {
  SelState state;
  unsigned long long count;
  unsigned keys[2 * kNoAllocMaxQ];
};
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[64] = {};

// Device address of g_noalloc_scratch on the current device, looked up once per
// device (host code only has a stand-in for the symbol, not its address).  The
// address belongs to the device's primary context: it is not looked up again
// after a cudaDeviceReset, which the header tells callers not to do.
int noalloc_scratch(NoAllocScratch** out) {
  int dev = 0;
  FSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FSG_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = static_cast<NoAllocScratch*>(g_noalloc_ptr[dev]);
  return FSG_OK;
}

}  // namespace
}  // namespace fsg

extern "C" int fsg_percentile_noalloc(const float* values_dev, int64_t n, int32_t abs_values, const double* q,
                                      int32_t nq, double* out, int64_t* nvalid, void* stream) {
  if ((n > 0 && !values_dev) || nq < 0 || (nq > 0 && (!q || !out))) return fail(FSG_ERR_INVALID, "null argument");
  if (nq > kNoAllocMaxQ)
    return fail(FSG_ERR_WORKSPACE, "fsg_percentile_noalloc takes at most %d percentiles per call, got %d",
                kNoAllocMaxQ, nq);
  for (int i = 0; i < nq; ++i)
    if (!(q[i] >= 0.0 && q[i] <= 100.0)) return fail(FSG_ERR_INVALID, "percentile %g outside [0, 100]", q[i]);
  cudaStream_t s = (cudaStream_t)stream;
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  NoAllocScratch* scr = nullptr;
  st = noalloc_scratch(&scr);
  if (st) return st;
  int grid = (int)std::max<long long>(1, std::min<long long>((n + NT - 1) / NT, (long long)di.sms * 8));
  FSG_CUDA(cudaMemsetAsync(&scr->count, 0, sizeof(unsigned long long), s));  // the array keeps the last call's data
  if (n > 0) {
    count_valid<<<grid, NT, 0, s>>>(values_dev, n, abs_values, &scr->count);
    FSG_LAUNCHED(1);
  }
  unsigned long long nv = 0;
  FSG_CUDA(cudaMemcpyAsync(&nv, &scr->count, sizeof(nv), cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  if (nvalid) *nvalid = (int64_t)nv;
  if (nv == 0) {
    for (int i = 0; i < nq; ++i) out[i] = std::nan("");
    return FSG_OK;
  }
  unsigned long long ranks[2 * kNoAllocMaxQ];
  LinearPick picks[kNoAllocMaxQ];
  int nr = 0;
  for (int i = 0; i < nq; ++i) {
    picks[i] = linear_pick((long long)nv, q[i]);
    ranks[nr++] = (unsigned long long)picks[i].lo;
    ranks[nr++] = (unsigned long long)picks[i].hi;
  }
  std::sort(ranks, ranks + nr);
  nr = (int)(std::unique(ranks, ranks + nr) - ranks);
  for (int r = 0; r < nr; ++r) {
    st = select_rank(values_dev, n, abs_values, ranks[r], &scr->state, grid, s);  // init_state clears the state
    if (st) return st;
    FSG_CUDA(cudaMemcpyAsync(&scr->keys[r], &scr->state.prefix, sizeof(unsigned), cudaMemcpyDeviceToDevice, s));
  }
  unsigned keys[2 * kNoAllocMaxQ];
  FSG_CUDA(cudaMemcpyAsync(keys, scr->keys, sizeof(unsigned) * nr, cudaMemcpyDeviceToHost, s));
  FSG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < nq; ++i) {
    int ia = (int)(std::lower_bound(ranks, ranks + nr, (unsigned long long)picks[i].lo) - ranks);
    int ib = (int)(std::lower_bound(ranks, ranks + nr, (unsigned long long)picks[i].hi) - ranks);
    out[i] = lerp_numpy(key_to_float(keys[ia]), key_to_float(keys[ib]), picks[i].gamma);
  }
  return FSG_OK;
}
