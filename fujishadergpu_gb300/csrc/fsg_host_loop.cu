// Host-buffer tile loop of the fused stencil: the single-device equivalent of
// process_dem_tiles' per-tile read -> H2D -> compute -> D2H cycle
// (core/tile_processor.py:822-1024, :1629-1683), with the three stages of
// consecutive batches overlapped.
//
// Consecutive tiles that form one row band of the grid (same core rows, cores
// side by side, one output offset) are one batch: the union of their windows
// goes down in one copy (one contiguous block when the band spans the
// raster's full width), one fsg_stencil call covers all of its tiles, and each
// plane's band of cores comes back in one copy.  Other tiles are batches of
// one.  Batches are assigned round-robin to NSLOT slots; each slot owns a
// device window buffer, one device buffer per requested plane and a stream,
// so the H2D copy of one batch, the kernels of the previous one and the D2H
// copies of the one before that run concurrently (separate copy engines for
// the two directions).  The slots' streams are ordered after, and joined back
// into, the caller's stream with events.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "fsg_common.cuh"

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

using namespace fsg;

extern "C" int fsg_stencil_host(const float* raster_host, int64_t ld, int32_t raster_h, int32_t raster_w,
                                const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                                const fsg_plane* planes_host, void* stream) {
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
  StreamScratch scratch;
  st = scratch.alloc(slot_bytes * nslot, caller);
  if (st) return st;
  FSG_CUDA(cudaEventRecord(S->start, caller));
  for (int i = 0; i < nslot; ++i) FSG_CUDA(cudaStreamWaitEvent(S->s[i], S->start, 0));
  int status = FSG_OK;
  std::vector<fsg_tile> local;
  for (size_t bi = 0; bi < batches.size() && status == FSG_OK; ++bi) {
    const Batch& B = batches[bi];
    if (B.ch == 0 || B.cw == 0) continue;
    const int k = (int)(bi % nslot);
    cudaStream_t s = S->s[k];
    char* base = static_cast<char*>(scratch.ptr) + slot_bytes * k;
    float* win = reinterpret_cast<float*>(base);
    // H2D: the window union (one contiguous block for a full-width band)
    const int64_t bpitch = (B.wx0 == 0 && B.ww == raster_w && ld == raster_w) ? (int64_t)raster_w : wpitch;
    cudaError_t e = cudaMemcpy2DAsync(win, bpitch * sizeof(float), raster_host + (int64_t)B.wy0 * ld + B.wx0,
                                      ld * sizeof(float), (size_t)B.ww * sizeof(float), B.wh,
                                      cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      status = cuda_fail(e, "cudaMemcpy2DAsync(H2D window)");
      break;
    }
    // kernels: the window union is a raster of its own; the core planes are dense band buffers
    fsg_plane dev_planes[FSG_STENCIL_NOUT];
    std::memset(dev_planes, 0, sizeof(dev_planes));
    char* p = base + (size_t)wpitch * maxwh * sizeof(float);
    int64_t opitch[FSG_STENCIL_NOUT] = {};
    for (int o : req) {
      dev_planes[o] = planes_host[o];
      dev_planes[o].ptr = p;
      // a full-width band of a full-width plane comes back as one contiguous block
      opitch[o] = (B.cw == planes_host[o].ld) ? (int64_t)B.cw : cpitch;
      dev_planes[o].ld = opitch[o];
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
    status = fsg_stencil(win, bpitch, B.wh, B.ww, local.data(), (int)local.size(), params, dev_planes, s);
    if (status) break;
    // D2H: the band of cores of every plane, into the caller's planes at (oy0, ox0)
    for (int o : req) {
      const size_t es = esize(planes_host[o].dtype);
      char* dst = static_cast<char*>(planes_host[o].ptr) + ((int64_t)B.oy0 * planes_host[o].ld + B.ox0) * es;
      e = cudaMemcpy2DAsync(dst, planes_host[o].ld * es, dev_planes[o].ptr, opitch[o] * es, (size_t)B.cw * es,
                            B.ch, cudaMemcpyDeviceToHost, s);
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
