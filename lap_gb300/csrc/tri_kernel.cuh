// tri_kernel.cuh -- sync-free sparse triangular solve over a level schedule.
//
// Replaces cusparseDcsrsv2_solve (cuda_blas.cu:731-820, :500, :516).  The
// rows are processed in the reference's natural ordering semantics -- every
// row is solved exactly as simple_lower/upper_triangular_solve
// (simple_blas.c:46-85) does: acc = rhs; acc -= l_ij * y_j in the row's
// column order; y_i = acc / d_i -- but the row-to-thread assignment follows a
// level schedule built on the host (TriPlan): warps hold rows of one level,
// so a warp never waits on itself, and blocks take a ticket at start so a
// block only ever waits on blocks that were scheduled before it (no
// deadlock whatever the residency).  There is no barrier between levels: a
// consumer spins on the producer's value (sentinel-initialised output), so
// the critical path costs one L2 round trip per level instead of a launch.
//
// OP supplies the right-hand side of a row and consumes the result, which is
// how the PCG fuses its vector updates and the r'w dot product into the
// solves.  OP contract:
//   void begin()                   every thread, at kernel start
//   bool active()                  false: skip all rows (converged solve)
//   T rhs(int row)                 right-hand side value of `row`
//   void done(int row, T y)        after y is published
//   void block_end(bid, nblocks, ticket, sm)
//                                  whole block, after its rows; must count
//                                  completion in ticket[1] and let the last
//                                  block reset ticket[0..1]
#pragma once

#include "gb_common.cuh"
#include "spmv_bundle.cuh"

namespace gb {

constexpr int kTriWarps = 8;      // warps per block
constexpr int kTriPrefetch = 8;   // dependencies held in registers before waiting

template <typename T>
struct TriArgs {
  int nwarps;
  const int* __restrict__ slot_row;
  const int* __restrict__ warp_ptr;
  const int* __restrict__ warp_len;
  const int* __restrict__ ecol;
  const T* __restrict__ eval;
  const T* __restrict__ diag;
  T* y;            // output, pre-filled with the sentinel
  unsigned* ticket; // [0] block order, [1] completion
  int* err;
};

__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

template <typename T, typename OP>
__global__ void __launch_bounds__(kTriWarps * 32) tri_solve_kernel(TriArgs<T> A, OP op) {
  __shared__ int s_bid;
  __shared__ double s_red[64];
  if (threadIdx.x == 0) s_bid = (int)atomicAdd(&A.ticket[0], 1u);
  op.begin();
  __syncthreads();
  const int bid = s_bid;
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = bid * kTriWarps + wid;
  if (op.active() && w < A.nwarps) {
    const int len = __ldg(A.warp_len + w);
    const int base = __ldg(A.warp_ptr + w);
    if (len >= 0) {
      // SHORT warp: one row per lane, dependencies column-major
      const int slot = w * 32 + lane;
      const int row = __ldg(A.slot_row + slot);
      if (row >= 0) {
        int cols[kTriPrefetch];
        T vals[kTriPrefetch];
#pragma unroll
        for (int k = 0; k < kTriPrefetch; ++k) {
          cols[k] = -1;
          vals[k] = T(0);
          if (k < len) {
            cols[k] = __ldg(A.ecol + base + k * 32 + lane);
            vals[k] = __ldg(A.eval + base + k * 32 + lane);
          }
        }
        const T dg = __ldg(A.diag + slot);
        T acc = op.rhs(row);
#pragma unroll
        for (int k = 0; k < kTriPrefetch; ++k)
          if (cols[k] >= 0) acc = sub_rn(acc, mul_rn(vals[k], wait_value(A.y + cols[k], A.err)));
        for (int k = kTriPrefetch; k < len; ++k) {
          const int c = __ldg(A.ecol + base + k * 32 + lane);
          if (c < 0) break;
          acc = sub_rn(acc, mul_rn(__ldg(A.eval + base + k * 32 + lane), wait_value(A.y + c, A.err)));
        }
        const T yv = publishable(div_rn(acc, dg));
        st_relaxed(A.y + row, yv);
        op.done(row, yv);
      }
    } else {
      // LONG warp: a single row with -len dependencies, reduced by the warp
      const int row = __ldg(A.slot_row + w * 32);
      const int cnt = -len;
      T s = T(0);
      for (int k = lane; k < cnt; k += 32) {
        const int c = __ldg(A.ecol + base + k);
        s = add_rn(s, mul_rn(__ldg(A.eval + base + k), wait_value(A.y + c, A.err)));
      }
      s = warp_sum(s);
      if (lane == 0) {
        const T yv = publishable(div_rn(sub_rn(op.rhs(row), s), __ldg(A.diag + w * 32)));
        st_relaxed(A.y + row, yv);
        op.done(row, yv);
      }
    }
  }
  op.block_end(bid, gridDim.x, A.ticket, s_red);
}

// Plain solve: rhs from an input vector.
template <typename T>
struct OpPlain {
  const T* __restrict__ x;
  __device__ __forceinline__ void begin() {}
  __device__ __forceinline__ bool active() const { return true; }
  __device__ __forceinline__ T rhs(int r) const { return x[r]; }
  __device__ __forceinline__ void done(int, T) {}
  __device__ __forceinline__ void block_end(int, int nblocks, unsigned* ticket, double*) {
    // the last block to finish resets the block-order ticket for the next launch
    if (threadIdx.x == 0) {
      __threadfence();
      if (atomicAdd(&ticket[1], 1u) == (unsigned)nblocks - 1u) {
        ticket[0] = 0u;
        ticket[1] = 0u;
        __threadfence();
      }
    }
  }
};

}  // namespace gb
