// gblap_internal.h -- internal structures shared by the libgblap translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <vector>

#include "gblap.h"

#define GB_CUDA_TRY(expr)                                                            \
  do {                                                                               \
    cudaError_t e_ = (expr);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      fprintf(stderr, "libgblap: %s failed at %s:%d: %s\n", #expr, __FILE__, __LINE__, \
              cudaGetErrorString(e_));                                               \
      return GB_CUDA_ERROR;                                                          \
    }                                                                                \
  } while (0)

#define GB_STR2(x) #x
#define GB_STR(x) GB_STR2(x)

#define GB_TRY(expr)             \
  do {                           \
    int s_ = (expr);             \
    if (s_ != GB_OK) return s_;  \
  } while (0)

namespace gb {

constexpr int kBundleRows = 32;   // rows per SpMV bundle (one warp)
constexpr int kBundleNnz = 512;   // products staged per bundle (4 KB FP64)
constexpr int kSpmvWarps = 8;     // warps per SpMV block
constexpr int kRedBlocksPerSM = 4;
constexpr int kRedThreads = 256;

// ----------------------------------------------------------- SpMV plan
// Rows are cut into bundles of <= kBundleRows rows whose entries fit the
// staging buffer; a single row with more entries is a "long" bundle that a
// whole warp reduces.  bundles[b] = first row of bundle b, bundles[nb] = n.
struct SpmvPlan {
  int n = 0, nnz = 0;
  int nbundles = 0;
  int *bundles = nullptr;   // device [nbundles+1]
  int long_rows = 0;        // diagnostics
  int rows_per_bundle = kBundleRows;
};

// ----------------------------------------------------------- triangular schedule
// Tiled level schedule of one triangular factor (see tri_kernel.cuh).  Rows
// are cut into contiguous tiles of tile_rows rows, processed in dependency
// order (ascending for a lower factor, descending for an upper one).  Inside
// a tile, rows are grouped by their global level (dependency depth in the
// whole factor), and each level into 32-row slices: a SHORT slice holds one row per lane with its
// dependencies column-major (entry k of lane l at ent + k*32 + l); a LONG
// slice holds one row with more than 32 dependencies, contiguous, reduced by
// a whole warp.
// Each level of a tile is stored as one or more RECORDS (tri_kernel.cuh):
// a 16-byte header, the rows, their diagonal and its reciprocal, and the
// dependency columns and values column-major -- contiguous and 16-byte
// aligned so one TMA bulk copy stages a record in shared memory.  The FP64
// and FP32 record buffers share the row partition; their value slots are
// written from the factor's value array through the fill maps.
struct RecordSet {
  unsigned char *buf = nullptr;  // records
  long long bytes = 0;
  long long *off = nullptr;      // [nrec] byte offset of each record
  int *nbytes = nullptr;         // [nrec]
  long long *vdst = nullptr;     // [nval] element index (T units) of each entry value
  long long *ddst = nullptr;     // [ndiag] element index of each diagonal
  long long *idst = nullptr;     // [ndiag] element index of each reciprocal
  void *long_val = nullptr;      // [nlong] values of long rows
};

struct TriPlan {
  int n = 0;
  bool lower = true;
  int nlevels = 0;           // global dependency depth (diagnostics)
  int tile_rows = 0;         // 0 in the levels form
  int ntiles = 0;
  // levels form: "tiles" are consecutive runs of records in global level
  // order with no rows of their own (every dependency is read through L2);
  // chosen when contiguous row tiles would hold few of the dependencies
  bool levels_form = false;
  int nlvl = 0;              // levels spanned by each tile, summed over tiles
  int nrec = 0;
  long long ndeps = 0;       // dependencies without padding (algorithmic size)
  int *tile_row0 = nullptr, *tile_row1 = nullptr;  // [ntiles], processing order
  int *tile_rec = nullptr;   // [ntiles+1]
  int *rec_flags = nullptr;  // [nrec]
  // r64: the factor's values as stored (the exact solves).  buf64s (FP64)
  // and r32 (FP32) hold the FMA form used inside the PCG: entry values
  // pre-multiplied by the reciprocal of their row's diagonal.  buf64s shares
  // r64's layout and offsets.
  RecordSet r64, r32;
  unsigned char* buf64s = nullptr;
  int nval = 0, ndiag = 0, nlong = 0;
  int *vsrc = nullptr;       // [nval] index of each entry value in the value source array
  int *dsrc = nullptr;       // [ndiag] index of each diagonal in the diagonal source array
  int *long_col = nullptr;   // [nlong]
  int *long_src = nullptr;   // [nlong]
  bool have32 = false;
  // every record is short with at most kTriHeld dependencies (no long rows,
  // hub parts or tail batches): the solve may run the SHORT kernel
  bool short_only = false;
  // r32 in the fixed record layout (short-only plans): read only by the
  // SHORT kernel; vdsrc[i] = the diagonal source index of value i's row
  bool fixed32 = false;
  int *vdsrc = nullptr;
  // rows in global level order, each level padded to a multiple of 32 with
  // -1 (the IC(0) factorization walks this order)
  int *order = nullptr;
  int norder = 0;
  unsigned *ticket = nullptr;  // [0] next tile, [1] finished tiles, [2] exited blocks
  // partial sums of split hub rows (one slot per partial record), FP64 and
  // FP32 views, held at the sentinel between uses
  int nslots = 0;
  double *part64 = nullptr;
  float *part32 = nullptr;
};

}  // namespace gb
