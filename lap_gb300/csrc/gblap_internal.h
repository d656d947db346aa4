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
// Rows are processed in level order (level = longest dependency chain), each
// level padded to whole warps so a warp never waits on itself.  A warp is
// either SHORT (32 rows, one per lane, dependencies stored column-major:
// entry k of lane l at ptr + k*32 + l) or LONG (one row, its dependencies
// contiguous, reduced by the whole warp).
struct TriPlan {
  int n = 0;
  bool lower = true;
  int nlevels = 0;
  int nwarps = 0;
  int nent = 0;
  long long ndeps = 0;       // dependencies without padding (algorithmic size)
  int *slot_row = nullptr;   // [nwarps*32] row or -1 (LONG warps: lane 0 only)
  int *warp_ptr = nullptr;   // [nwarps+1] entry offsets
  int *warp_len = nullptr;   // [nwarps] deps per lane (SHORT) or deps of the row (LONG, negated)
  int *ecol = nullptr;       // [nent] dependency row, -1 padding
  int *emap = nullptr;       // [nent] index of the value in the entry source array
  int *dmap = nullptr;       // [nwarps*32] index of the diagonal in the diagonal source array
  double *eval = nullptr;    // [nent]
  double *diag = nullptr;    // [nwarps*32]
  float *eval32 = nullptr;
  float *diag32 = nullptr;
  unsigned *ticket = nullptr;  // dynamic block order + completion counter
};

}  // namespace gb
