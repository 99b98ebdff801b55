/*
 * fsg.h -- C ABI of libfsg.so, the GB300 (sm_103a) raster hot path of
 * FujiShaderGPU: fused 3x3-class stencils (hillshade / slope / curvature),
 * the multiscale topousm_fast unsharp mask, openness ray-marching, FP64
 * order statistics and the integer output encoding.
 *
 * Conventions
 *   - Every pointer named `*_dev` or documented as "device" is CUDA device
 *     memory owned by the caller; the library never frees it.  Host structs
 *     (tile lists, parameter blocks) are read during the call only.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *     All work is stream-ordered: a call returns once its kernels are queued.
 *   - Rasters are row-major float32 with NaN as NoData; `ld` is the row pitch
 *     in elements.  Coordinates are (row, col) = (y, x), 0-based.
 *   - Return value: FSG_OK (0) or a negative FSG_ERR_* code.  A human-readable
 *     message for the last error on the calling thread is fsg_last_error().
 *
 * Each entry point names the reference interface it replaces, as a path:line
 * inside the FujiShaderGPU source tree.
 */
#ifndef FSG_H_
#define FSG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSG_ABI_VERSION 1

/* ---------------------------------------------------------------- status */
enum fsg_status {
  FSG_OK = 0,
  FSG_ERR_INVALID = -1,     /* bad argument: null pointer, bad size, core outside window (ValueError) */
  FSG_ERR_SHAPE = -2,       /* window < 3 px along an axis: np.gradient(edge_order=2) raises ValueError */
  FSG_ERR_DTYPE = -3,       /* unsupported output dtype */
  FSG_ERR_CUDA = -4,        /* a CUDA runtime call failed */
  FSG_ERR_TIMEOUT = -5,     /* a bounded device-side wait ran out; the kernel returned early */
  FSG_ERR_ABORTED = -6,     /* a tile in a queue reported an error; see the per-tile status */
  FSG_ERR_WORKSPACE = -7,   /* caller workspace too small / scratch over its maximum */
  FSG_ERR_UNSUPPORTED = -8  /* combination not supported (e.g. no CUDA device) */
};

/* ----------------------------------------------------------- output planes */
enum fsg_dtype { FSG_F32 = 0, FSG_U8 = 1, FSG_I16 = 2 };

/* Output plane of a kernel.  Pixel (y, x) of a tile core is written at
 * ptr[(out_y0 + y - core_y0) * ld + (out_x0 + x - core_x0)] (see fsg_tile).
 * For FSG_U8/FSG_I16 the value is encoded as
 *   DN = clip(rint(q_a * v + q_b), q_min, q_max), non-finite v -> 0
 * (io/output_encoding.py:178-190; q_a/q_b from quantize_params :130-175).
 * fsg_stencil / fsg_stencil_host require [q_min, q_max] inside the type's range
 * ([0, 255] for FSG_U8, [-32768, 32767] for FSG_I16; FSG_ERR_INVALID otherwise). */
typedef struct fsg_plane {
  void* ptr;          /* device pointer; NULL = output not requested */
  int64_t ld;         /* elements per row */
  int32_t dtype;      /* enum fsg_dtype */
  int32_t reserved;
  float q_a, q_b;
  int32_t q_min, q_max;
} fsg_plane;

/* One tile of the reference tile loop (core/tile_processor.py:1610-1627):
 * the window (core + clipped halo) is what the reference block function sees,
 * so its edges carry the edge rules (np.gradient edge_order=2, 'nearest' /
 * 'reflect' filter modes); only the core is written. */
typedef struct fsg_tile {
  int32_t win_y0, win_x0, win_h, win_w;      /* raster coords */
  int32_t core_y0, core_x0, core_h, core_w;  /* raster coords, inside the window */
  int32_t out_y0, out_x0;                    /* plane coords of the core's first pixel */
  int32_t reserved0, reserved1;
  double pixel_scale_x, pixel_scale_y;       /* signed metres per pixel (tile_processor.py:910-932) */
} fsg_tile;

/* ------------------------------------------------------------------ plans
 * A plan is one entry point's call prepared once: its tile tables are
 * uploaded into device memory the plan owns, so fsg_plan_launch issues only
 * kernels, memsets and device-side copies on the given stream and can be
 * captured into a CUDA graph (the core/ tile scheduler's persistent work
 * queue, core/tile_processor.py:1629-1683, replayed as one graph launch).
 * The buffers named at creation must stay valid while the plan is used.
 * Creating and destroying a plan synchronise; launching does not. */
typedef struct fsg_plan fsg_plan;
int fsg_plan_launch(fsg_plan* plan, void* stream);
void fsg_plan_destroy(fsg_plan* plan);

/* ------------------------------------------------------------- utilities */
int fsg_abi_version(void);
const char* fsg_version(void);
const char* fsg_last_error(void);
/* Number of kernels launched by this library on the calling process (all devices). */
int64_t fsg_launch_count(void);
/* Device-side timing of the dominant kernel of each call (the fused stencil's
 * streaming pass, the topousm_fast strip pass, the openness ray-march): between
 * fsg_timing_begin and fsg_timing_end, up to max_launches such launches are
 * bracketed by CUDA events on their stream; fsg_timing_end synchronises those
 * events and returns the summed kernel time.  No reference counterpart
 * (measurement support for the roofline figures). */
int fsg_timing_begin(int32_t max_launches);
int fsg_timing_end(double* total_ms, int32_t* launches);
/* Device-side failures since the last call, cleared on read (synchronises): bit 0 = the
 * fused stencil's streaming pass gave up waiting for a tensor-memory copy (its outputs
 * are then incomplete); bit 1 = the tensor-core topousm_fast kernel gave up waiting on
 * one of its pipeline barriers (its tiles are then incomplete).  No reference
 * counterpart. */
int fsg_kernel_errors(uint32_t* flags);
/* Scratch memory.  Entry points that need scratch take it stream-ordered from a
 * memory pool the library creates per device; up to 16 GiB of freed scratch stays
 * in the pool for the next call (the device's default pool would hand it back at
 * every synchronisation and map it again on the next call).  This returns the
 * pool's high-water mark of bytes in use on the current device since the last
 * reset (reset != 0: then starts a new one).  No reference counterpart. */
int fsg_scratch_high_water(uint64_t* bytes, int32_t reset);

/* NoData mask (core/tile_processor.py:185-196): mask_dev[i] = 1 where
 * isnan(v) or (has_nodata and (|v - nodata| <= 1e-6 in float32, or v == nodata)). */
int fsg_nodata_mask(const float* raster_dev, int64_t ld, int32_t h, int32_t w,
                    double nodata, int32_t has_nodata, uint8_t* mask_dev, int64_t mask_ld,
                    void* stream);

/* ------------------------------------------------------- fused stencils */
enum fsg_stencil_out {
  FSG_OUT_HILLSHADE = 0,     /* algorithms/_impl_hillshade.py:20-54 */
  FSG_OUT_SLOPE = 1,         /* algorithms/_impl_slope.py:19-35 */
  FSG_OUT_CURV_MEAN = 2,     /* algorithms/_impl_curvature.py:19-57, curvature_type='mean' */
  FSG_OUT_CURV_GAUSSIAN = 3,
  FSG_OUT_CURV_PLANFORM = 4,
  FSG_OUT_CURV_PROFILE = 5,
  FSG_OUT_DX = 6,            /* dz/dx of handle_nan_for_gradient (_nan_utils.py:50-74), float32 */
  FSG_OUT_DY = 7,            /* dz/dy of handle_nan_for_gradient, float32 */
  FSG_STENCIL_NOUT = 8
};
enum fsg_slope_unit { FSG_SLOPE_DEGREE = 0, FSG_SLOPE_PERCENT = 1, FSG_SLOPE_RADIAN = 2 };

typedef struct fsg_stencil_params {
  double azimuth;       /* degrees (default 315) */
  double altitude;      /* degrees (default 45) */
  double z_factor;      /* hillshade vertical exaggeration (default 1) */
  double pixel_size;    /* fallback step when |pixel_scale| < 1e-9 */
  double nodata;        /* NoData sentinel, used when has_nodata != 0 */
  int32_t has_nodata;
  int32_t slope_unit;   /* enum fsg_slope_unit */
} fsg_stencil_params;

/* One fused pass over a list of tiles: reads each halo window once and writes
 * every requested plane of planes[FSG_STENCIL_NOUT] (ptr NULL = skip).
 * Replaces, per tile, handle_nan_for_gradient (_nan_utils.py:50-74) followed by
 * compute_hillshade_block / compute_slope_block / compute_curvature_block, the
 * NoData re-mask (core/tile_compute.py:132-152) and quantize_array
 * (io/output_encoding.py:178-190), as called from process_single_tile
 * (core/tile_processor.py:822-1024) via algorithms/tile/dask_bridge.py:72-151. */
int fsg_stencil(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                const fsg_plane* planes, void* stream);
/* fsg_stencil prepared as a plan (same arguments, no stream). */
int fsg_stencil_plan(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                     const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                     const fsg_plane* planes, fsg_plan** plan);

/* The same fused pass over a raster and output planes in HOST memory (pinned
 * memory gives asynchronous copies): per tile, the window is copied to the
 * device, the kernels run, and every requested core is copied back into the
 * host planes at (out_y0, out_x0); three tiles are in flight at once (H2D /
 * compute / D2H overlapped on library-owned streams ordered after `stream`;
 * `stream` waits for all of them).  Replaces the per-tile read -> cp.asarray ->
 * block function -> cp.asnumpy cycle of process_single_tile
 * (core/tile_processor.py:851-996) driven by process_dem_tiles' executor
 * (:1629-1683).  Host buffers must stay valid until `stream` completes. */
int fsg_stencil_host(const float* raster_host, int64_t ld, int32_t raster_h, int32_t raster_w,
                     const fsg_tile* tiles, int32_t ntiles, const fsg_stencil_params* params,
                     const fsg_plane* planes_host, void* stream);

/* ------------------------------------------------------------ topousm_fast */
typedef struct fsg_topousm_params {
  /* Small radii computed per window (algorithms/_impl_topousm_fast.py:49-100) with
   * their absolute weights (not renormalised after the large-radius split,
   * _impl_topousm_fast.py:113-130).  nradii may be 0 when only the coarse field
   * contributes. */
  const int32_t* radii;
  const double* weights;
  int32_t nradii;
  int32_t has_nodata;
  double pixel_size;        /* drives the per-radius decimation factor (_nan_utils.py:555-601) */
  double nodata;
  /* Large radii from one global overview field (dask_bridge.py:237-249):
   * result += w_large * z - bilinear(field at global pixel centres).  coarse_dev
   * NULL = no large part.  full_h/full_w: the raster the field spans; each
   * tile's global origin is its window origin. */
  const float* coarse_dev;
  int64_t coarse_ld;
  int32_t coarse_h, coarse_w;
  int64_t full_h, full_w;
  double w_large;
  /* p99(|raw|) divisor (_normalization.py:35-41); 0 = write the raw sum. */
  double scale;
  /* Arithmetic of the full-resolution box means (no reference counterpart):
   * FSG_TOPOUSM_EXACT = 64-bit fixed-point running sums on the CUDA cores;
   * FSG_TOPOUSM_TENSOR = banded Toeplitz products on the tcgen05 tensor cores in
   * split BF16 (three terms per FP32 operand, FP32 accumulation) for windows
   * without NoData, the exact kernel for tiles that hold NoData.  The tensor path
   * applies to at most 4 full-resolution radii, each 2..32 (else: exact). */
  int32_t path;
} fsg_topousm_params;

enum fsg_topousm_path { FSG_TOPOUSM_EXACT = 0, FSG_TOPOUSM_TENSOR = 1 };

/* topousm_fast over a list of tiles; writes each core into `out` (float32 or
 * int16/uint8 codes).  Replaces, per tile, dask_bridge._direct_topousm_fast
 * (algorithms/tile/dask_bridge.py:225-271) = compute_topousm_fast_efficient_block
 * + the large-radius part + apply_global_normalization, and quantize_array. */
int fsg_topousm(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                const fsg_tile* tiles, int32_t ntiles, const fsg_topousm_params* params,
                const fsg_plane* out, void* stream);
/* fsg_topousm prepared as a plan (same arguments, no stream); radius lists
 * that take the fused strip pass only (ascending, full-resolution radii first),
 * else FSG_ERR_UNSUPPORTED. */
int fsg_topousm_plan(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                     const fsg_tile* tiles, int32_t ntiles, const fsg_topousm_params* p,
                     const fsg_plane* out, fsg_plan** plan);

/* Large-radius field on the overview grid: sum_i f32(w_i) * mean_{r_i}(coarse), r_i =
 * max(1, round(radius_i / decimation)) -- compute_topousm_fast_large_coarse_field
 * (algorithms/_impl_topousm_fast.py:133-155). */
int fsg_topousm_coarse_field(const float* coarse_dev, int64_t ld, int32_t h, int32_t w,
                             const int32_t* radii, const double* weights, int32_t n,
                             double decimation, float* field_dev, int64_t field_ld, void* stream);

/* Overview DEM for the coarse field: NaN-aware mean of the source pixels whose
 * centres fall in each output cell (an exact block mean for integer factors).
 * Stands in for the GDAL average-resampled overview read of
 * core/tile_processor.py:575-585. */
int fsg_overview(const float* raster_dev, int64_t ld, int32_t h, int32_t w, double nodata,
                 int32_t has_nodata, float* out_dev, int32_t out_h, int32_t out_w, int64_t out_ld,
                 void* stream);

/* _radius_to_downsample_factor(radius, pixel_size, 'topousm_fast') (_nan_utils.py:555-601). */
int fsg_topousm_downsample_factor(double radius, double pixel_size);

/* --------------------------------------------------------------- statistics */
/* numpy.percentile(v[~isnan(v)], q, method='linear') of float32 device data
 * (|v| when abs_values != 0): exact order statistics by radix select, FP64
 * interpolation.  Writes nq doubles to host `out` (NaN if no valid value) and
 * the valid count to *nvalid (may be NULL).  Synchronises `stream`.
 * Replaces cp.percentile in topousm_fast_stat_func (_normalization.py:21-32) and
 * robust_unsigned_stretch_stat_func (_global_stats.py:181-203). */
int fsg_percentile(const float* values_dev, int64_t n, int32_t abs_values, const double* q, int32_t nq,
                   double* out, int64_t* nvalid, void* stream);

/* One pass of the radix select behind fsg_percentile, for statistics merged
 * across devices (a raster sharded over GPUs): the histogram of the
 * order-preserving uint32 keys of the valid float32 values (|v| when
 * abs_values != 0) whose bits under `mask` equal `prefix`, binned by
 * (key >> shift) & (2^bits - 1), bits <= 11.  Writes 2^bits counts to host
 * `hist_out`; synchronises `stream`.  Summing the histograms of all shards
 * and picking bins identically on every rank selects the exact order
 * statistics of the union (no counterpart in the reference, which runs the
 * statistics on one device). */
int fsg_key_histogram(const float* values_dev, int64_t n, int32_t abs_values, uint32_t prefix, uint32_t mask,
                      int32_t shift, int32_t bits, uint64_t* hist_out, void* stream);

/* Population standard deviation of the valid (non-NaN) values, FP64
 * (the fallback scale of _normalization.py:30).  Synchronises `stream`. */
int fsg_std(const float* values_dev, int64_t n, double* out, void* stream);

/* Same result as fsg_percentile, but allocates nothing.  It has no counterpart in
 * the reference.  It is for callers that cannot allocate device memory during a
 * run: an application whose GPU memory is owned and budgeted by its own pool, or
 * a latency-critical caller that cannot accept the implicit device
 * synchronisation cudaMalloc / cudaFree may cause.  Its scratch (~17 KB) is a
 * fixed array that every GPU loading libfsg.so holds until the process exits.
 * Limits: at most 16 percentiles per call (nq > 16 -> FSG_ERR_WORKSPACE); any n.
 * The first call on a device looks up the array's device address (once per
 * device, with that device current).  The address stays valid for the life of
 * the device's primary context: do not call it again after cudaDeviceReset on
 * that device.  All calls share the one array: calls that overlap on the GPU
 * (other streams, other host threads) race and must be serialised by the
 * caller.  It synchronises `stream` (twice), so it cannot be captured into a
 * CUDA graph. */
int fsg_percentile_noalloc(const float* values_dev, int64_t n, int32_t abs_values, const double* q, int32_t nq,
                           double* out, int64_t* nvalid, void* stream);

/* ----------------------------------------------------------------- encoding */
/* out = (v - offset) / scale in float32 (scale <= 0: unchanged), max(., 0) when
 * clamp_min0, NaN kept; stored as float32 or int16/uint8 codes.  Replaces
 * apply_global_normalization (_global_stats.py:123-153) with
 * topousm_fast_norm_func (_normalization.py:35-41), the openness display
 * stretch (algorithms/tile/dask_bridge.py:173-187) and quantize_array
 * (io/output_encoding.py:178-190). */
int fsg_affine(const float* in_dev, int64_t ld, int32_t h, int32_t w, double offset, double scale,
               int32_t clamp_min0, const fsg_plane* out, void* stream);

/* ------------------------------------------------------------------ openness */
enum fsg_openness_mode {
  FSG_OPENNESS_REFERENCE = 0,  /* 10 sampled distances per ray (_impl_openness.py:65-68) */
  FSG_OPENNESS_DENSE = 1       /* every pixel step r = 1..max_distance */
};

typedef struct fsg_openness_params {
  int32_t openness_type;    /* 0 positive, 1 negative */
  int32_t num_directions;   /* default 16 */
  int32_t max_distance;     /* pixels, default 50 */
  int32_t mode;             /* enum fsg_openness_mode */
  double pixel_size;        /* fallback when |pixel_scale| < 1e-9 */
  double nodata;
  int32_t has_nodata;
  int32_t reserved;
  double stretch_lo, stretch_scale;  /* display stretch (p1, p99 - p1); scale <= 1e-12: none */
} fsg_openness_params;

/* Exact openness ray-march over a list of tiles.  `display` receives
 * ((mean/(pi/2)) clipped to [0,1])^(1/2.2) (then the optional stretch) as float32
 * or int16/uint8 codes; `raw_deg_dev` (nullable, float32, same addressing as the
 * display plane, row pitch raw_ld) receives the directional mean angle in
 * degrees.  Replaces compute_openness_vectorized
 * (algorithms/_impl_openness.py:31-132) and _direct_openness
 * (algorithms/tile/dask_bridge.py:208-222). */
int fsg_openness(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                 const fsg_tile* tiles, int32_t ntiles, const fsg_openness_params* params,
                 const fsg_plane* display, float* raw_deg_dev, int64_t raw_ld, void* stream);
/* fsg_openness prepared as a plan (same arguments, no stream). */
int fsg_openness_plan(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                      const fsg_tile* tiles, int32_t ntiles, const fsg_openness_params* params,
                      const fsg_plane* display, float* raw_deg_dev, int64_t raw_ld, fsg_plan** plan);

/* ------------------------------------------------------- ambient occlusion */
typedef struct fsg_ao_params {
  int32_t num_samples;      /* directions per ring, default 16 */
  int32_t has_nodata;
  double radius;            /* pixels, default 10 */
  double intensity;         /* default 1 */
  double pixel_size;        /* fallback when |pixel_scale| < 1e-9 */
  double nodata;
  double stretch_lo, stretch_scale;  /* display stretch (p1, p99 - p1); scale <= 1e-12: none */
} fsg_ao_params;

/* Ambient occlusion over a list of tiles: per window, 4 rings x num_samples
 * edge-padded samples, clamped elevation angle weighted by the ring's distance
 * factor, AO = clip(1 - mean * intensity, 0, 1), Gaussian sigma 1 ('nearest'
 * at the window edge), ^(1/2.2), NaN at NoData, optional stretch, written as
 * float32 or int16/uint8 codes to `out` at the cores.  Replaces
 * compute_ambient_occlusion_block (algorithms/_impl_ambient_occlusion.py:32-121)
 * called per tile by _direct_ambient_occlusion
 * (algorithms/tile/dask_bridge.py:190-203). */
int fsg_ambient_occlusion(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                          const fsg_tile* tiles, int32_t ntiles, const fsg_ao_params* params,
                          const fsg_plane* out, void* stream);
/* fsg_ambient_occlusion prepared as a plan (same arguments, no stream). */
int fsg_ambient_occlusion_plan(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                               const fsg_tile* tiles, int32_t ntiles, const fsg_ao_params* params,
                               const fsg_plane* out, fsg_plan** plan);

/* Host-only: the ray offsets the kernel uses (dx, dy per sample, directions in
 * order; ray_len[d] samples for direction d).  Returns FSG_ERR_WORKSPACE with
 * ray_len filled if `capacity` is too small. */
int fsg_openness_offsets(int32_t num_directions, int32_t max_distance, int32_t mode, int32_t* ox, int32_t* oy,
                         int32_t* ray_len, int32_t capacity);

/* --------------------------------------------------------------- prepare */
/* The NoData detection and void fill of preprocess_dem_to_cog
 * (io/dem_preprocess.py:462-726) on in-memory device rasters; the GDAL / COG
 * file I/O around it is not part of this library. */
enum fsg_fill_mode { FSG_FILL_NONE = 0, FSG_FILL_ENCLOSED = 1, FSG_FILL_ALL = 2 };

/* Nearest-neighbour read of the raster at oh x ow (source index
 * trunc((i + 0.5) * n / o) per axis; stands in for GDAL's NEAREST read,
 * io/dem_preprocess.py:540-546) and, when declared_dev is not NULL, its
 * declared-NoData mask (value == nodata, or NaN for a NaN nodata). */
int fsg_nearest_sample(const float* raster_dev, int64_t ld, int32_t h, int32_t w, int32_t oh, int32_t ow,
                       double nodata, int32_t has_nodata, float* sample_dev, int64_t sample_ld,
                       uint8_t* declared_dev, int64_t declared_ld, void* stream);

/* _nan_aware_coarse_average (io/dem_preprocess.py:135-188) of a (ch k) x (cw k)
 * sample: a sample is NoData when declared, non-finite or equal (as float32) to
 * one of nodata_values (at most 16); coarse = float32(sum / count) of the valid
 * samples (0 for a void), valid = count > 0; *any_void (nullable, synchronises)
 * tells whether some cell is a void. */
int fsg_coarse_average(const float* sample_dev, int64_t ld, const uint8_t* declared_dev, int64_t declared_ld,
                       int32_t ch, int32_t cw, int32_t k, const double* nodata_values, int32_t n_values,
                       float* coarse_dev, int64_t coarse_ld, uint8_t* valid_dev, int64_t valid_ld,
                       int32_t* any_void, void* stream);

/* The value statistics of _detect_sentinel_nodata (io/dem_preprocess.py:241-275)
 * over the finite, undeclared samples: their number, smallest and largest value,
 * and, when some value holds at least min_fraction of them, the most frequent
 * value (the smallest on ties) and its count (*mode_count = 0 otherwise).
 * -0 and +0 count as one value.  FSG_ERR_UNSUPPORTED when more than 4096
 * 16-bit key bins reach min_fraction (min_fraction far below 1 / 4096).
 * Synchronises. */
int fsg_value_mode(const float* sample_dev, int64_t ld, int32_t h, int32_t w, const uint8_t* declared_dev,
                   int64_t declared_ld, double min_fraction, int64_t* n_finite, double* vmin, double* vmax,
                   double* mode_value, int64_t* mode_count, void* stream);

/* Number of samples equal (as float32) to value.  Synchronises. */
int fsg_count_equal(const float* sample_dev, int64_t ld, int32_t h, int32_t w, double value, int64_t* count,
                    void* stream);

/* pushpull_fill (algorithms/_pyramid_fill.py:24-84): a fully finite surface,
 * valid cells kept exactly (synchronises once per push level). */
int fsg_pushpull_fill(const float* coarse_dev, int64_t coarse_ld, const uint8_t* valid_dev, int64_t valid_ld,
                      int32_t h, int32_t w, float* out_dev, int64_t out_ld, void* stream);

/* _edge_connected_mask (utils/nodata_handler.py:13-25): the mask cells
 * 4-connected to a border cell of the mask (the mask: cells != 0, or == 0 with
 * invert set); synchronises per pass. */
int fsg_edge_connected(const uint8_t* mask_dev, int64_t mask_ld, int32_t h, int32_t w, int32_t invert,
                       uint8_t* out_dev, int64_t out_ld, void* stream);

/* _apply_band_fill + _sample_coarse (io/dem_preprocess.py:729-826) over rows
 * [row0, row0 + rows) of the raster: NoData (declared, non-finite, one of
 * extra_nodata) -> NaN; with a fill mode and a surface, NoData cells take the
 * bilinear ('nearest') sample of the ch x cw surface at ((y + 0.5) ch/h - 0.5,
 * (x + 0.5) cw/w - 0.5) in float32, except, for FSG_FILL_ENCLOSED, where the
 * bilinear exterior mask exceeds 0.5.  Row r goes to out + (r - row0) * out_ld
 * (out may be the raster itself).  *nonfinite (nullable, synchronises): with
 * FSG_FILL_ALL, some cell stayed non-finite. */
int fsg_fill_apply(const float* raster_dev, int64_t ld, int32_t h, int32_t w, int32_t row0, int32_t rows,
                   double nodata, int32_t has_nodata, const double* extra_nodata, int32_t n_extra,
                   int32_t fill_mode, const float* surface_dev, int64_t surface_ld, const uint8_t* exterior_dev,
                   int64_t exterior_ld, int32_t ch, int32_t cw, float* out_dev, int64_t out_ld, int32_t* nonfinite,
                   void* stream);

/* ------------------------------------------------------------- spatial mode */
/* _smooth_for_radius(block, radius, pixel_size, algorithm)
 * (algorithms/_nan_utils.py:527-552): identity for radius <= 1, else the
 * NaN-aware Gaussian (sigma = max(0.5, r/2), 'nearest'), or for large radii the
 * NaN-aware f x f block mean, Gaussian at that resolution and bilinear zoom
 * back.  algorithm_factor is the per-algorithm factor of the decimation rule
 * (_nan_utils.py:571-581): 1.0 hillshade and slope, 1.1 curvature, 1.15
 * topousm_fast, 1.4 openness.  src and dst are h x w float32 device arrays
 * (NaN = NoData) that must not overlap. */
int fsg_smooth(const float* src, int64_t ld, int32_t h, int32_t w, double radius, double pixel_size,
               double algorithm_factor, float* dst, int64_t dst_ld, void* stream);

/* _downsample_nan_aware(block, f) (algorithms/_nan_utils.py:604-668): the
 * NaN-aware f x f block mean summed in NumPy's float32 order, enclosed voids
 * filled by the normalised Gaussian; dst is ceil(h/f) x ceil(w/f). */
int fsg_downsample_nan_aware(const float* src, int64_t ld, int32_t h, int32_t w, int32_t f, float* dst,
                             int64_t dst_ld, void* stream);

/* _upsample_to_shape(block, (th, tw)) (algorithms/_nan_utils.py:671-698):
 * scipy's zoom(order=1, mode='nearest') in float64, NaN-aware when the source
 * holds NaN, last row / column repeated where the zoom is smaller; writes the
 * target region [y0, y0+oh) x [x0, x0+ow) to dst. */
int fsg_upsample_to_shape(const float* src, int64_t ld, int32_t h, int32_t w, int32_t th, int32_t tw, int32_t y0,
                          int32_t x0, int32_t oh, int32_t ow, float* dst, int64_t dst_ld, void* stream);

/* The raster window [y0, y0+h) x [x0, x0+w) mirrored by `depth` samples on
 * every side, repeating the edge sample (dask map_overlap boundary='reflect',
 * as the Dask branch of the spatial products uses it,
 * algorithms/_nan_utils.py:500-512), NoData -> NaN.  dst is
 * (h + 2 depth) x (w + 2 depth); depth <= min(h, w). */
int fsg_pad_reflect(const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w, int32_t y0,
                    int32_t x0, int32_t h, int32_t w, int32_t depth, double nodata, int32_t has_nodata,
                    float* dst, int64_t dst_ld, void* stream);

/* acc = src * weight (first != 0) or acc + src * weight, float32 without a fused
 * multiply-add: one step of the weighted combination of per-radius responses
 * (_combine_multiscale_dask, algorithms/_nan_utils.py:182-213). */
int fsg_accumulate(const float* src, int64_t ld, int32_t h, int32_t w, float weight, int32_t first,
                   float* acc, int64_t acc_ld, void* stream);

/* Combination step of per-radius responses (_combine_multiscale_dask,
 * algorithms/_nan_utils.py:182-213; _impl_hillshade.py:109-131):
 * FSG_COMBINE_WSUM as fsg_accumulate (weight 1: the plain sum), FSG_COMBINE_MAX /
 * FSG_COMBINE_MIN the element-wise extreme with NaN propagating as in NumPy's
 * max / min over the stack; first != 0 starts the combination with src. */
enum fsg_combine_op { FSG_COMBINE_WSUM = 0, FSG_COMBINE_MAX = 1, FSG_COMBINE_MIN = 2 };
int fsg_combine(const float* src, int64_t ld, int32_t h, int32_t w, int32_t op, float weight, int32_t first,
                float* acc, int64_t acc_ld, void* stream);

/* One large-radius response of a tile: the coarse (overview) response sampled
 * bilinearly at global pixel centres (_bilinear_sample_coarse,
 * algorithms/_nan_utils.py:255-281) for the raster region
 * [y0, y0+h) x [x0, x0+w), whose first pixel has the global coordinates
 * (gy0, gx0) in a full_h x full_w raster (full sizes < 2^24); NaN where the
 * raster region is NoData (:395); accumulated into acc as fsg_accumulate does. */
int fsg_sample_coarse_accumulate(const float* coarse_dev, int64_t cld, int32_t ch, int32_t cw,
                                 const float* raster_dev, int64_t ld, int32_t raster_h, int32_t raster_w,
                                 int32_t y0, int32_t x0, int32_t h, int32_t w, int64_t gy0, int64_t gx0,
                                 int64_t full_h, int64_t full_w, double nodata, int32_t has_nodata, float weight,
                                 int32_t first, float* acc, int64_t acc_ld, void* stream);

/* The last steps of a combined response before its store: divided by
 * `divisor` (the plain mean's count; 1 for none), then, with
 * stretch_scale > 1e-12, the display stretch max((v - stretch_lo) /
 * stretch_scale, 0) of apply_display_stretch_dask
 * (algorithms/_global_stats.py:156-178), NaN kept.  keep_nodata_values != 0
 * skips the NoData mask (the window-level process() of the reference returns
 * the combined responses unmasked). */
typedef struct fsg_store_finish {
  float divisor;
  float stretch_lo;
  float stretch_scale;
  int32_t keep_nodata_values;
} fsg_store_finish;

/* Store of a combined tile core: NaN where the raster region
 * [gy0, gy0+h) x [gx0, gx0+w) is NoData (apply_nodata_mask,
 * core/tile_compute.py:132-152) unless finish says otherwise, the finishing
 * steps (finish may be NULL: mask only), then the plane's encoding; `out`
 * addresses the region's first pixel. */
int fsg_masked_store(const float* acc, int64_t acc_ld, const float* raster_dev, int64_t ld, int32_t raster_h,
                     int32_t raster_w, int32_t gy0, int32_t gx0, int32_t h, int32_t w, double nodata,
                     int32_t has_nodata, const fsg_store_finish* finish, const fsg_plane* out, void* stream);

/* ------------------------------------------------------ openness surrogate */
/* Kernels of the convolutional openness surrogate (no counterpart in the
 * reference, which runs the exact ray-march only).  Feature maps are float32
 * [batch][h][w][channels], channels fastest; w a multiple of 16.  Weights of a
 * 3x3 layer are float32 w[9][cin][32] (tap = 3*ky + kx), packed once into a
 * BF16 table of 9 * cin_pad/16 * 256 uint32 (cin_pad = 16 for cin <= 16, else
 * 32); `transpose` packs the table of the data gradient (cin == 32). */
int fsg_conv_pack_weights(const float* w_dev, int32_t cin, int32_t transpose, uint32_t* wb_dev, void* stream);

/* y = relu?(conv3x3_dil(x) + bias) (+ res): implicit GEMM on the tensor cores
 * (BF16 operands, FP32 accumulation).  flip mirrors the taps (with a transposed
 * table: the data gradient).  bias and res may be NULL. */
int fsg_conv3x3(const float* x_dev, int32_t cin_pad, int32_t batch, int32_t h, int32_t w, int32_t dil,
                const uint32_t* wb_dev, const float* bias_dev, int32_t relu, int32_t flip, const float* res_dev,
                float* y_dev, void* stream);

/* dw[9][cin][32] += sum over pixels of x(p + tap*dil)[ci] * gz(p)[co] (atomic; zero dw first). */
int fsg_conv3x3_wgrad(const float* x_dev, int32_t cin, int32_t cin_pad, int32_t batch, int32_t h, int32_t w,
                      int32_t dil, const float* gz_dev, float* dw_dev, void* stream);

/* 1x1 head over 32 channels: out[p] = sum_c h[p][c] w[c] + bias. */
int fsg_head_forward(const float* h_dev, const float* w_dev, float bias, int64_t npix, float* out_dev,
                     void* stream);

/* Head gradients: gh = gout * w (+ gres); gw[c] += sum_p h[p][c] gout[p]; gb += sum_p gout[p]
 * (gw, gb accumulated atomically; gres may be NULL). */
int fsg_head_backward(const float* h_dev, const float* w_dev, const float* gout_dev, const float* gres_dev,
                      int64_t npix, float* gh_dev, float* gw_dev, float* gb_dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FSG_H_ */
