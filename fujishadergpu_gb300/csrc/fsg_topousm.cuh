// Tables shared by the topousm_fast kernels (fsg_topousm.cu: the CUDA-core
// strip kernels and the per-window decimation; fsg_topousm_tc.cu: the
// tensor-core box means): one tile's window and decimated grids, the strip
// work items and the launch arguments of the strip kernels.
#pragma once

#include <vector>

#include "fsg_filters.cuh"

namespace fsg {

constexpr int ST_NT = 256, ST_G = 8, ST_SEG = 8, ST_MAXR = 64, ST_MAXN = 6, ST_MAXD = 4;

struct DecK {       // one decimated radius of a tile
  const float* ms;  // its coarse mean (ROW_MEAN output), row pitch w
  int h, w;
  double zy, zx;    // corner-aligned zoom factors (in - 1) / (out - 1)
  float weight;
};

struct TopoTileK {
  ZView z;                 // the window
  int cy0, cx0, ch, cw;    // core, window coordinates
  int gy0, gx0;            // global coordinates of the window origin
  char* out;               // output plane at the core origin
  const int* nan_flag;     // NoData anywhere in the window
  DecK dec[ST_MAXD];
  int ndec;
};

struct StripItem {
  int tile, x0, y0, y1;    // output columns [x0, x0 + TW) (window), rows [y0, y1)
};

struct StripArgs {
  const TopoTileK* tiles;
  const StripItem* items;
  int nitems;
  int nr, R, TW;
  int radii[ST_MAXN];
  float weights[ST_MAXN];
  float fn[ST_MAXN], rn[ST_MAXN];  // box size 2r+1 and RN(1/(2r+1))
  const float* field;      // large-radius field (nullable)
  long long fld;
  int fh, fw;
  float sy, sx, w_large, scale;
  float rscale;            // RN(1 / scale)
  long long old;
  int dtype;
  float qa, qb;
  int qmin, qmax;
  int have_small;
  int ring;                // topousm_fixed: rows of the prefix ring (2R + 2G + 1)
  const unsigned* zmax;    // topousm_fixed: max |z| over the windows (float bits)
  const int* nitems_dev;   // topousm_fixed / topousm_hybrid: item count on the device (overrides nitems)
};

// Tensor-core box means of the full-resolution radii (fsg_topousm_tc.cu): at
// most TC_MAXNR radii, each 2..32.  tc_prepare copies the epilogue fields of
// S; tc_bind points the arguments at the device tables; tc_items lists the CTA
// tiles (128 rows x 192 columns) of every core; tc_launch queues the kernel.
// Tiles whose input region holds NoData are appended to fix_items /
// fix_count (StripItems of 192 columns) for the exact kernels.
constexpr int TC_MAXNR = 4;
struct TcArgs;
int tc_supported(const int* radii, int nfull);
int tc_prepare(TcArgs** out, const StripArgs& S, int nfull, size_t* smem);
void tc_bind(TcArgs* A, const TopoTileK* tiles, const int4* items, int nitems, StripItem* fix_items, int* fix_count,
             unsigned* zmax);
void tc_items(const TopoTileK* tk, int ntiles, std::vector<int4>* items);
int tc_launch(const TcArgs* A, size_t smem, cudaStream_t s);
void tc_release(TcArgs* A);
int tc_take_errors(unsigned* flags);

}  // namespace fsg
