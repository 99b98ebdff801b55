// Host-buffer tile loop of the fused stencil: the single-device equivalent of
// process_dem_tiles' per-tile read -> H2D -> compute -> D2H cycle
// (core/tile_processor.py:822-1024, :1629-1683), with the three stages of
// consecutive tiles overlapped.
//
// Tiles are assigned round-robin to NSLOT slots; each slot owns a device
// window buffer, one device core buffer per requested plane and a stream, so
// the H2D copy of one tile, the kernels of the previous one and the D2H copies
// of the one before that run concurrently (separate copy engines for the two
// directions).  The slots' streams are ordered after, and joined back into,
// the caller's stream with events.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "fsg_common.cuh"

namespace fsg {
namespace {

constexpr int NSLOT = 3;

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

}  // namespace
}  // namespace fsg

using namespace fsg;

extern "C" int fsg_stencil_host(const float* raster_host, int64_t ld, int32_t raster_h, int32_t raster_w,
                                const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                                const fsg_plane* planes_host, void* stream) {
  if (!raster_host || !params || !planes_host || (ntiles > 0 && !tiles)) return fail(FSG_ERR_INVALID, "null argument");
  if (ntiles < 0 || raster_h < 0 || raster_w < 0 || ld < raster_w) return fail(FSG_ERR_INVALID, "bad raster shape");
  int st = validate_tiles(raster_h, raster_w, tiles, ntiles, 3);
  if (st) return st;
  int maxwh = 0, maxww = 0, maxch = 0, maxcw = 0;
  for (int t = 0; t < ntiles; ++t) {
    maxwh = std::max(maxwh, tiles[t].win_h);
    maxww = std::max(maxww, tiles[t].win_w);
    maxch = std::max(maxch, tiles[t].core_h);
    maxcw = std::max(maxcw, tiles[t].core_w);
  }
  if (ntiles == 0 || maxch == 0 || maxcw == 0) return FSG_OK;
  const int64_t wpitch = ((int64_t)maxww + 31) & ~(int64_t)31;  // elements, 128-byte rows
  std::vector<int> req;
  for (int o = 0; o < FSG_STENCIL_NOUT; ++o)
    if (planes_host[o].ptr) {
      if (planes_host[o].dtype < FSG_F32 || planes_host[o].dtype > FSG_I16)
        return fail(FSG_ERR_DTYPE, "plane %d: dtype %d", o, planes_host[o].dtype);
      req.push_back(o);
    }
  if (req.empty()) return fail(FSG_ERR_INVALID, "no output plane requested");
  const int64_t cpitch = ((int64_t)maxcw + 127) & ~(int64_t)127;  // elements of each core plane row
  size_t slot_bytes = (size_t)wpitch * maxwh * sizeof(float);
  for (int o : req) slot_bytes += (size_t)cpitch * maxch * esize(planes_host[o].dtype) + 256;
  slot_bytes = (slot_bytes + 255) & ~(size_t)255;
  cudaStream_t caller = (cudaStream_t)stream;
  SlotStreams* S = nullptr;
  st = slot_streams(&S);
  if (st) return st;
  StreamScratch scratch;
  st = scratch.alloc(slot_bytes * NSLOT, caller);
  if (st) return st;
  FSG_CUDA(cudaEventRecord(S->start, caller));
  for (int i = 0; i < NSLOT; ++i) FSG_CUDA(cudaStreamWaitEvent(S->s[i], S->start, 0));
  int status = FSG_OK;
  for (int t = 0; t < ntiles && status == FSG_OK; ++t) {
    const fsg_tile& T = tiles[t];
    if (T.core_h == 0 || T.core_w == 0) continue;
    const int k = t % NSLOT;
    cudaStream_t s = S->s[k];
    char* base = static_cast<char*>(scratch.ptr) + slot_bytes * k;
    float* win = reinterpret_cast<float*>(base);
    // H2D: the tile window
    cudaError_t e = cudaMemcpy2DAsync(win, wpitch * sizeof(float), raster_host + (int64_t)T.win_y0 * ld + T.win_x0,
                                      ld * sizeof(float), (size_t)T.win_w * sizeof(float), T.win_h,
                                      cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      status = cuda_fail(e, "cudaMemcpy2DAsync(H2D window)");
      break;
    }
    // kernels: the window is a raster of its own; the core planes are dense buffers
    fsg_plane dev_planes[FSG_STENCIL_NOUT];
    std::memset(dev_planes, 0, sizeof(dev_planes));
    char* p = base + (size_t)wpitch * maxwh * sizeof(float);
    for (int o : req) {
      dev_planes[o] = planes_host[o];
      dev_planes[o].ptr = p;
      dev_planes[o].ld = cpitch;
      p += ((size_t)cpitch * maxch * esize(planes_host[o].dtype) + 255) & ~(size_t)255;
    }
    fsg_tile local = T;
    local.win_y0 = 0;
    local.win_x0 = 0;
    local.core_y0 = T.core_y0 - T.win_y0;
    local.core_x0 = T.core_x0 - T.win_x0;
    local.out_y0 = 0;
    local.out_x0 = 0;
    status = fsg_stencil(win, wpitch, T.win_h, T.win_w, &local, 1, params, dev_planes, s);
    if (status) break;
    // D2H: the core of every plane, into the caller's planes at (out_y0, out_x0)
    for (int o : req) {
      const size_t es = esize(planes_host[o].dtype);
      char* dst = static_cast<char*>(planes_host[o].ptr) + ((int64_t)T.out_y0 * planes_host[o].ld + T.out_x0) * es;
      e = cudaMemcpy2DAsync(dst, planes_host[o].ld * es, dev_planes[o].ptr, cpitch * es, (size_t)T.core_w * es,
                            T.core_h, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) {
        status = cuda_fail(e, "cudaMemcpy2DAsync(D2H plane)");
        break;
      }
    }
  }
  for (int i = 0; i < NSLOT; ++i) {
    cudaEventRecord(S->done[i], S->s[i]);
    cudaStreamWaitEvent(caller, S->done[i], 0);
  }
  return status;
}
