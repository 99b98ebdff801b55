// libfsg.so runtime: version, thread-local error messages, launch accounting,
// device properties and the NoData mask kernel.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fsg_common.cuh"

namespace fsg {

namespace {
thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};
std::mutex g_dev_mutex;
DeviceInfo g_dev_cache[64];
// device-side timing of marked kernels (fsg_timing_begin / fsg_timing_end)
std::mutex g_tmu;
std::atomic<bool> g_timing{false};
std::vector<cudaEvent_t> g_tev;
int g_tn = 0;
}  // namespace

void timing_mark(cudaStream_t s, bool start) {
  if (!g_timing.load(std::memory_order_relaxed)) return;
  std::lock_guard<std::mutex> lk(g_tmu);
  const int n = (int)g_tev.size();
  if (start ? (g_tn % 2 != 0 || g_tn + 2 > n) : (g_tn % 2 != 1)) return;
  if (cudaEventRecord(g_tev[g_tn], s) == cudaSuccess) ++g_tn;
}

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(FSG_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

void count_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int device_info(DeviceInfo* out) {
  int dev = 0;
  FSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FSG_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  DeviceInfo& d = g_dev_cache[dev];
  if (d.device != dev) {
    int sms = 0, optin = 0, per_sm = 0;
    FSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FSG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    FSG_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    d.sms = sms;
    d.smem_optin = (size_t)optin;
    d.smem_per_sm = (size_t)per_sm;
    d.device = dev;
  }
  *out = d;
  return FSG_OK;
}

// The library's stream-ordered scratch pool of a device.  The device's default
// pool hands its free memory back to the driver at every synchronisation (its
// release threshold is 0), so a caller that synchronises between calls paid for
// mapping the scratch again on each call: with the host-buffer stencil's ~5 GB
// of staging at 16384^2 that doubled the call (55 against 24 ms).  This pool
// keeps up to kScratchKeep bytes of freed scratch for the next call.
constexpr uint64_t kScratchKeep = 16ull << 30;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[64] = {};

int scratch_pool(cudaMemPool_t* out) {
  int dev = 0;
  FSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FSG_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_pool_mutex);
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    FSG_CUDA(cudaMemPoolCreate(&p, &props));
    uint64_t keep = kScratchKeep;
    FSG_CUDA(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pools[dev] = p;
  }
  *out = g_pools[dev];
  return FSG_OK;
}

// Host-to-device copies of a call's tables through pinned staging.  From pageable
// memory the driver may synchronise with the stream to stage a copy, so a call waited
// for all the work already queued on its stream (the previous call's) before it could
// queue its own: back-to-back calls of the host-buffer stencil never overlapped.  From
// pinned memory the copy is queued like any other.  A per-device ring of kStageSlots
// pinned slots, each reused once the copy that last read it has run (its event), each
// grown on demand.
namespace {
constexpr int kStageSlots = 32;
struct StageSlot {
  void* p = nullptr;
  size_t cap = 0;
  cudaEvent_t ev = nullptr;
  bool pending = false;
};
struct StageRing {
  StageSlot slot[kStageSlots];
  int next = 0;
};
std::mutex g_stage_mutex;
StageRing g_stage[64];
}  // namespace

int upload_async(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return FSG_OK;
  // a captured copy would read the slot when the graph replays, after later calls reused
  // it: direct calls are not capturable (the fsg_*_plan entry points are)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  FSG_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(FSG_ERR_UNSUPPORTED, "tile tables cannot be uploaded inside a stream capture: capture a plan's launch");
  int dev = 0;
  FSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FSG_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_stage_mutex);
  StageRing& R = g_stage[dev];
  StageSlot& k = R.slot[R.next];
  R.next = (R.next + 1) % kStageSlots;
  if (k.pending) {
    FSG_CUDA(cudaEventSynchronize(k.ev));
    k.pending = false;
  }
  if (!k.ev) FSG_CUDA(cudaEventCreateWithFlags(&k.ev, cudaEventDisableTiming));
  if (k.cap < bytes) {
    if (k.p) {
      FSG_CUDA(cudaFreeHost(k.p));
      k.p = nullptr;
      k.cap = 0;
    }
    const size_t cap = (std::max<size_t>(bytes, (size_t)64 << 10) + 4095) & ~(size_t)4095;
    FSG_CUDA(cudaHostAlloc(&k.p, cap, cudaHostAllocDefault));
    k.cap = cap;
  }
  std::memcpy(k.p, src, bytes);
  FSG_CUDA(cudaMemcpyAsync(dst, k.p, bytes, cudaMemcpyHostToDevice, s));
  FSG_CUDA(cudaEventRecord(k.ev, s));
  k.pending = true;
  return FSG_OK;
}

namespace {
__global__ void nodata_mask_kernel(const float* __restrict__ r, long long ld, int h, int w, float ndf,
                                   int has_nodata, uint8_t* __restrict__ m, long long mld) {
  long long n = (long long)h * w;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    long long y = i / w, x = i - y * w;
    m[y * mld + x] = is_nodata(__ldg(r + y * ld + x), ndf, has_nodata != 0) ? 1 : 0;
  }
}
}  // namespace

}  // namespace fsg

extern "C" {

int fsg_abi_version(void) { return FSG_ABI_VERSION; }

int fsg_scratch_high_water(uint64_t* bytes, int32_t reset) {
  if (!bytes) return fsg::fail(FSG_ERR_INVALID, "null argument");
  cudaMemPool_t p = nullptr;
  int st = fsg::scratch_pool(&p);
  if (st) return st;
  uint64_t v = 0;
  FSG_CUDA(cudaMemPoolGetAttribute(p, cudaMemPoolAttrUsedMemHigh, &v));
  *bytes = v;
  if (reset) {
    uint64_t z = 0;
    FSG_CUDA(cudaMemPoolSetAttribute(p, cudaMemPoolAttrUsedMemHigh, &z));
  }
  return FSG_OK;
}

const char* fsg_version(void) { return "fsg-gb300 0.1.0 (sm_103a)"; }

const char* fsg_last_error(void) { return fsg::g_last_error.c_str(); }

int64_t fsg_launch_count(void) { return fsg::g_launches.load(); }

int fsg_plan_launch(fsg_plan* plan, void* stream) {
  if (!plan) return fsg::fail(FSG_ERR_INVALID, "null plan");
  return plan->launch((cudaStream_t)stream);
}

void fsg_plan_destroy(fsg_plan* plan) { delete plan; }

int fsg_timing_begin(int32_t max_launches) {
  using namespace fsg;
  if (max_launches < 1 || max_launches > 1 << 16) return fail(FSG_ERR_INVALID, "max_launches %d", max_launches);
  std::lock_guard<std::mutex> lk(g_tmu);
  for (cudaEvent_t e : g_tev) cudaEventDestroy(e);
  g_tev.assign((size_t)2 * max_launches, nullptr);
  for (auto& e : g_tev) FSG_CUDA(cudaEventCreate(&e));
  g_tn = 0;
  g_timing.store(true);
  return FSG_OK;
}

int fsg_timing_end(double* total_ms, int32_t* launches) {
  using namespace fsg;
  if (!total_ms || !launches) return fail(FSG_ERR_INVALID, "null argument");
  g_timing.store(false);
  std::lock_guard<std::mutex> lk(g_tmu);
  double tot = 0.0;
  const int pairs = g_tn / 2;
  for (int i = 0; i < pairs; ++i) {
    FSG_CUDA(cudaEventSynchronize(g_tev[2 * i + 1]));
    float ms = 0.f;
    FSG_CUDA(cudaEventElapsedTime(&ms, g_tev[2 * i], g_tev[2 * i + 1]));
    tot += ms;
  }
  *total_ms = tot;
  *launches = pairs;
  g_tn = 0;
  return FSG_OK;
}

int fsg_nodata_mask(const float* raster_dev, int64_t ld, int32_t h, int32_t w, double nodata,
                    int32_t has_nodata, uint8_t* mask_dev, int64_t mask_ld, void* stream) {
  using namespace fsg;
  if (h < 0 || w < 0) return fail(FSG_ERR_INVALID, "negative raster shape %d x %d", h, w);
  if ((long long)h * w == 0) return FSG_OK;
  if (!raster_dev || !mask_dev) return fail(FSG_ERR_INVALID, "null pointer");
  if (ld < w || mask_ld < w) return fail(FSG_ERR_INVALID, "row pitch smaller than width");
  DeviceInfo di;
  int st = device_info(&di);
  if (st) return st;
  long long n = (long long)h * w;
  int blocks = (int)std::min<long long>((n + 255) / 256, (long long)di.sms * 8);
  nodata_mask_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(raster_dev, ld, h, w, (float)nodata,
                                                               has_nodata, mask_dev, mask_ld);
  FSG_LAUNCHED(1);
  return FSG_OK;
}

}  // extern "C"
