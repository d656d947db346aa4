// tri_kernel.cuh -- tiled sync-free sparse triangular solve.
//
// Replaces cusparseDcsrsv2_solve (cuda_blas.cu:731-820, :500, :516).  Every
// row is solved as simple_lower/upper_triangular_solve (simple_blas.c:46-85)
// does: acc = rhs; acc -= l_ij * y_j in the row's column order; y_i = acc /
// d_i.  EXACT keeps that rounding (separate mul and sub, a true division);
// otherwise the row uses FMAs and the precomputed reciprocal of d_i -- GB300
// runs FP64 at 1/64 of its FP32 rate, so every FP64 instruction on the
// dependency chain counts.
//
// Schedule (TriPlan, built on the host): rows are cut into contiguous tiles;
// inside a tile, rows are grouped by their level with respect to the tile's
// own rows, and each level into 32-row slices (entries column-major).  One
// CTA solves one tile at a time, holding the tile's values in shared memory:
//   A) rhs of every row into shared memory      (coalesced, tile-wide)
//   B) level by level: each warp solves slices of the level; a dependency
//      inside the tile is read from shared memory (ready after the previous
//      level's barrier), one in an earlier tile is read from global memory,
//      spinning on the producer's value (outputs are pre-filled with a
//      sentinel) with __nanosleep backoff; results go to shared memory and
//      global memory; __syncthreads between levels
//   C) per-row epilogue (fused vector updates, dot partials), coalesced.
// The next level's slice (indices, values, first remote values) is loaded
// before each barrier, so the dependency chain does not wait on DRAM.
// Tiles are taken by ticket in dependency order by a persistent grid, so a
// tile only ever waits on tiles already being solved by running CTAs.
//
// OP contract:
//   void begin();  bool active();  void inactive_end()   (block 0, !active)
//   T rhs(int row);                 phase A
//   void done(int row, T y);        phase C
//   void chunk_end(tile_ix, ntiles, ticket, sm)   whole block, after the
//        tile; ticket[1] counts finished tiles (chunk_finished()).
#pragma once

#include "gb_common.cuh"
#include "kernels.h"
#include "spmv_bundle.cuh"

namespace gb {

constexpr int kTriThreads = 128;  // 4 warps per CTA
constexpr int kTriPrefetch = 8;   // dependencies held in registers per row

template <typename T>
struct TriArgs {
  int ntiles;
  const int* __restrict__ tile_row0;   // [ntiles] first row (processing order)
  const int* __restrict__ tile_row1;   // [ntiles] one past the last row
  const int* __restrict__ tile_lvl;    // [ntiles+1] level range of each tile
  const int* __restrict__ lvl_slice;   // [nlevels_total+1] slice range of each level
  const int* __restrict__ slice_rows;  // [nslices*32] row or -1
  const int* __restrict__ slice_ent;   // [nslices] entry offset
  const int* __restrict__ slice_len;   // [nslices] deps per lane, or -deps of a long row
  const int* __restrict__ ecol;        // [nent] dependency row or -1
  const T* __restrict__ eval;
  const T* __restrict__ diag;          // [nslices*32]
  const T* __restrict__ dinv;          // [nslices*32] 1/diag
  T* y;              // output, pre-filled with the sentinel
  unsigned* ticket;  // [0] next tile, [1] finished tiles, [2] exited blocks
  int* err;
  int lower;
};

__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

// Counts a finished tile; true in the block that finished the last one.
// Thread 0 only, after the tile's partials are written.
__device__ __forceinline__ bool chunk_finished(unsigned* ticket, int nchunks) {
  __threadfence();
  return atomicAdd(&ticket[1], 1u) == (unsigned)nchunks - 1u;
}

// One slice's registers: a row per lane and its first kTriPrefetch deps.
template <typename T>
struct SliceRegs {
  int row, len, base;
  int cols[kTriPrefetch];
  T vals[kTriPrefetch];
  T rem[kTriPrefetch];  // early-read remote values (may still be the sentinel)
  T dg;
};

template <typename T>
__device__ __forceinline__ void load_slice(const TriArgs<T>& A, int s, int lane, int t0, int t1,
                                           SliceRegs<T>& R, bool exact) {
  R.len = __ldg(A.slice_len + s);
  R.base = __ldg(A.slice_ent + s);
  R.row = __ldg(A.slice_rows + s * 32 + lane);
  if (R.len < 0 || R.row < 0) return;
  R.dg = exact ? __ldg(A.diag + s * 32 + lane) : __ldg(A.dinv + s * 32 + lane);
#pragma unroll
  for (int k = 0; k < kTriPrefetch; ++k) {
    R.cols[k] = -1;
    if (k < R.len) {
      const int c = __ldg(A.ecol + R.base + k * 32 + lane);
      R.cols[k] = c;
      R.vals[k] = __ldg(A.eval + R.base + k * 32 + lane);
      if (c >= 0 && (c < t0 || c >= t1)) R.rem[k] = ld_relaxed(A.y + c);
    }
  }
}

template <typename T>
__device__ __forceinline__ T dep_value(const TriArgs<T>& A, const T* sm, int c, int t0, int t1,
                                       T early) {
  if (c >= t0 && c < t1) return sm[c - t0];
  if (!is_sentinel(early)) return early;
  return wait_value(A.y + c, A.err);
}

template <typename T, bool EXACT>
__device__ __forceinline__ void solve_slice(const TriArgs<T>& A, T* sm, int t0, int t1,
                                            const SliceRegs<T>& R, int lane) {
  if (R.row < 0) return;
  T acc = sm[R.row - t0];
#pragma unroll
  for (int k = 0; k < kTriPrefetch; ++k) {
    const int c = R.cols[k];
    if (c >= 0) {
      const T v = dep_value(A, sm, c, t0, t1, R.rem[k]);
      acc = EXACT ? sub_rn(acc, mul_rn(R.vals[k], v)) : fma_rn(-R.vals[k], v, acc);
    }
  }
  for (int k = kTriPrefetch; k < R.len; ++k) {
    const int c = __ldg(A.ecol + R.base + k * 32 + lane);
    if (c < 0) break;
    const T l = __ldg(A.eval + R.base + k * 32 + lane);
    const T v = dep_value(A, sm, c, t0, t1, sentinel<T>());
    acc = EXACT ? sub_rn(acc, mul_rn(l, v)) : fma_rn(-l, v, acc);
  }
  const T yv = publishable(EXACT ? div_rn(acc, R.dg) : acc * R.dg);
  sm[R.row - t0] = yv;
  st_relaxed(A.y + R.row, yv);
}

// A row with more than 32 dependencies: the whole warp reduces it.
template <typename T, bool EXACT>
__device__ __forceinline__ void solve_long(const TriArgs<T>& A, T* sm, int t0, int t1, int s,
                                           int lane) {
  const int row = __ldg(A.slice_rows + s * 32);
  const int cnt = -__ldg(A.slice_len + s);
  const int base = __ldg(A.slice_ent + s);
  T acc = T(0);
  for (int k = lane; k < cnt; k += 32) {
    const int c = __ldg(A.ecol + base + k);
    const T v = dep_value(A, sm, c, t0, t1, sentinel<T>());
    acc = add_rn(acc, mul_rn(__ldg(A.eval + base + k), v));
  }
  acc = warp_sum(acc);
  if (lane == 0) {
    const T r = sub_rn(sm[row - t0], acc);
    const T yv = publishable(EXACT ? div_rn(r, __ldg(A.diag + s * 32)) : r * __ldg(A.dinv + s * 32));
    sm[row - t0] = yv;
    st_relaxed(A.y + row, yv);
  }
}

template <typename T, typename OP, bool EXACT>
__global__ void __launch_bounds__(kTriThreads) tri_tile_kernel(TriArgs<T> A, OP op) {
  extern __shared__ __align__(16) unsigned char tri_smem[];
  T* sm = reinterpret_cast<T*>(tri_smem);
  __shared__ int s_tile;
  __shared__ double s_red[64];
  op.begin();
  if (!op.active()) {
    if (blockIdx.x == 0 && threadIdx.x == 0) op.inactive_end();
    return;  // no ticket touched
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int W = kTriThreads / 32;
  while (true) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(&A.ticket[0], 1u);
    __syncthreads();
    const int k = s_tile;
    __syncthreads();
    if (k >= A.ntiles) break;
    const int t0 = __ldg(A.tile_row0 + k), t1 = __ldg(A.tile_row1 + k);
    // A) right-hand sides
    for (int i = t0 + threadIdx.x; i < t1; i += kTriThreads) sm[i - t0] = op.rhs(i);
    const int l0 = __ldg(A.tile_lvl + k), l1 = __ldg(A.tile_lvl + k + 1);
    SliceRegs<T> R;
    bool have = false;
    if (l0 < l1) {
      const int s = __ldg(A.lvl_slice + l0) + wid;
      if (s < __ldg(A.lvl_slice + l0 + 1)) {
        load_slice(A, s, lane, t0, t1, R, EXACT);
        have = true;
      }
    }
    __syncthreads();
    // B) levels of the tile
    for (int lv = l0; lv < l1; ++lv) {
      const int s0 = __ldg(A.lvl_slice + lv), s1 = __ldg(A.lvl_slice + lv + 1);
      for (int s = s0 + wid; s < s1; s += W) {
        if (!have) load_slice(A, s, lane, t0, t1, R, EXACT);
        have = false;
        if (R.len < 0) solve_long<T, EXACT>(A, sm, t0, t1, s, lane);
        else solve_slice<T, EXACT>(A, sm, t0, t1, R, lane);
      }
      if (lv + 1 < l1) {
        const int sn = s1 + wid;  // this warp's first slice of the next level
        if (sn < __ldg(A.lvl_slice + lv + 2)) {
          load_slice(A, sn, lane, t0, t1, R, EXACT);
          have = true;
        }
      }
      __syncthreads();
    }
    // C) epilogue
    for (int i = t0 + threadIdx.x; i < t1; i += kTriThreads) op.done(i, sm[i - t0]);
    op.chunk_end(k, A.ntiles, A.ticket, s_red);
    __syncthreads();
  }
  // the last block to leave resets the counters for the next launch
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&A.ticket[2], 1u) == gridDim.x - 1u) {
      A.ticket[0] = 0u;
      A.ticket[1] = 0u;
      A.ticket[2] = 0u;
      __threadfence();
    }
  }
}

int tri_blocks_per_sm();

// Launches the tiled solve: dynamic shared memory = one tile of T values; a
// persistent grid of min(tiles, SMs x resident CTAs) blocks.
template <typename T, typename OP, bool EXACT>
int tri_launch(const TriPlan& p, const TriArgs<T>& A, OP op, cudaStream_t s) {
  if (p.ntiles <= 0) return GB_OK;
  const size_t smem = (size_t)p.tile_rows * sizeof(T);
  static bool attr_set = false;  // one per instantiation
  if (!attr_set) {
    GB_CUDA_TRY(cudaFuncSetAttribute(tri_tile_kernel<T, OP, EXACT>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    attr_set = true;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tri_tile_kernel<T, OP, EXACT>,
                                                    kTriThreads, smem) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  per_sm = per_sm < tri_blocks_per_sm() ? per_sm : tri_blocks_per_sm();
  const long long cap = (long long)device_sm_count() * per_sm;
  const int grid = (int)(p.ntiles < cap ? p.ntiles : cap);
  tri_tile_kernel<T, OP, EXACT><<<grid, kTriThreads, smem, s>>>(A, op);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

template <typename T>
TriArgs<T> tri_args(const TriPlan& p, T* y, int* err);

// Plain solve: rhs from an input vector.
template <typename T>
struct OpPlain {
  const T* __restrict__ x;
  __device__ __forceinline__ void begin() {}
  __device__ __forceinline__ bool active() const { return true; }
  __device__ __forceinline__ void inactive_end() {}
  __device__ __forceinline__ T rhs(int r) const { return x[r]; }
  __device__ __forceinline__ void done(int, T) {}
  __device__ __forceinline__ void chunk_end(int, int nchunks, unsigned* ticket, double*) {
    if (threadIdx.x == 0) chunk_finished(ticket, nchunks);
  }
};

}  // namespace gb
