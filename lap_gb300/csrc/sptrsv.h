// sptrsv.h -- level schedules for the sync-free triangular solves and IC(0).
#pragma once

#include <vector>

#include "gblap_internal.h"

namespace gb {

// Dependency description of one triangular factor, in summation order:
// row i depends on dep_col[row_ptr[i] .. row_ptr[i+1]) whose values live at
// ent_src[dep_src[..]]; its diagonal at diag_src_arr[diag_src[i]].
struct TriDeps {
  int n = 0;
  bool lower = true;
  std::vector<int> row_ptr, dep_col, dep_src, diag_src;
};

// LAP GPU convention: diagonal stored inside the factor (last in an L row,
// first in a U row, but found anywhere in the row).  Returns GB_BAD_INPUT
// when a row has no diagonal or a dependency on the wrong side.
int deps_embedded(int n, const int* ia, const int* ja, bool lower, TriDeps* d);
// LAP CPU convention: strict factor, diagonal in a separate array (index i).
int deps_strict(int n, const int* ia, const int* ja, bool lower, TriDeps* d);
// IC(0) on A's full pattern: lower = A's strict-lower entries, upper = L^T
// read through the transpose positions; values come from the factor stored
// on A's pattern.  tpos[k] = index of entry (j, i) for entry k = (i, j).
int transpose_positions(int n, const int* ia, const int* ja, std::vector<int>* tpos);
int deps_ichol(int n, const int* ia, const int* ja, const std::vector<int>& tpos, bool lower,
               TriDeps* d);

// tile_rows <= 0: one tile per SM for large matrices, 1024..16384 rows.
// Tiles of more than kTriMaxTileRows64 rows (up to kTriMaxTileRows32) fit
// shared memory only as FP32 and may be solved in FP32 only.
constexpr int kTriMaxTileRows64 = 16384;
constexpr int kTriMaxTileRows32 = 32768;
// level_run: records per run in the levels form (0: one per consumer warp
// of an FP64 CTA; FP32 plans pass tri_consumer_warps(4))
int tri_plan_build(const TriDeps& d, TriPlan* plan, int tile_rows = 0, int level_run = 0);
// consumer warps of one triangular-solve CTA for elements of elem_bytes
int tri_consumer_warps(int elem_bytes);
int tri_default_tile_rows(int n);
// Tile rows of the FP32 plans: the FP64 default, or GBLAP_TRI_TILE_ROWS32.
int tri_default_tile_rows32(int n);
// Resident CTAs per SM of the tiled solves (default 1, limited by shared
// memory anyway); GBLAP_TRI_BLOCKS_PER_SM overrides it (1..8).
int tri_grid(int ntiles);
int tri_blocks_per_sm();
void tri_set_blocks_per_sm(int bps);
void tri_plan_free(TriPlan* plan);
// Writes the record values from value arrays: always the exact FP64 records;
// kFillFma64 adds the FMA-form FP64 copy, kFillFma32 the FMA-form FP32
// records (what the PCG's FP64 / FP32 solves read).
enum { kFillExact = 0, kFillFma64 = 1, kFillFma32 = 2 };
int tri_plan_fill(TriPlan* plan, const double* ent_src, const double* diag_src, int mode,
                  cudaStream_t s);

// y = T^{-1} x with the plan's values, rounded as the reference rounds.  y
// must not alias x.
int tri_solve_plain(const TriPlan* plan, const double* x, double* y, int* err, cudaStream_t s);

// IC(0) factorization on A's pattern (left-looking, sync-free, level order
// of the lower schedule).  f receives the factor in symmetric storage: the
// strict-lower entries hold L, the diagonal sqrt pivots, the strict upper
// L^T.  zero_pivot (device int) receives the first offending row + 1 or 0.
int ichol_factor_dev(int n, const int* ia, const int* ja, const double* a, const int* dpos,
                     const int* tpos, const TriPlan* lower_plan, double* f, int* done,
                     unsigned* ticket, int* zero_pivot, int* err, cudaStream_t s);

}  // namespace gb
