// spmv_bundle.cuh -- CSR SpMV over row bundles (one warp per bundle).
//
// A bundle is up to 32 consecutive rows whose entries fit a per-warp staging
// buffer.  Phase 1: the warp walks the bundle's contiguous entry range with
// coalesced loads of ja/a (4 entries per lane in flight) and stages either
// the products (alpha*a_j)*x(ja_j) (EXACT) or just the gathered x(ja_j) in
// shared memory.  Phase 2: lane l sums row l's entries in column order.
//
// EXACT reproduces LAP's simple_csr_matvec (simple_blas.c:24-44) bit for
// bit: y = beta*y, then y += (alpha*a_j)*x_j left to right with separate
// round-to-nearest multiply and add (the reference's gcc build does not
// contract them).  Otherwise alpha must be 1 and each entry costs one FMA --
// on GB300 FP64 runs at 1/64 of the FP32 rate, so the fused PCG kernels use
// this form.  A row with more than kBundleNnz entries is reduced by the
// whole warp (lane-strided partial sums, then a shuffle tree: same value up
// to summation order).
//
// The x operand and the per-row epilogue are functors, so the PCG kernels
// fuse their vector updates and dot products into the SpMV.
#pragma once

#include "gb_common.cuh"

namespace gb {

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Epilogue contract:
//   T init(int row)           -> starting value of the row sum (beta*y or 0)
//   void store(int row, T v)  -> consume the finished row value
// X contract:
//   T operator()(int col)     -> x value at col
//
// bundles == nullptr selects the plan-free layout: bundle b is rows
// [32b, 32b+32); one whose entries overflow the staging buffer is walked row
// by row with the whole warp.
template <typename T, bool EXACT, typename XF, typename EP>
__device__ __forceinline__ void spmv_bundle(int b, int n, const int* __restrict__ bundles,
                                            const int* __restrict__ ia,
                                            const int* __restrict__ ja,
                                            const T* __restrict__ a, T alpha, XF& xf, EP& ep,
                                            T* stage) {
  const int lane = threadIdx.x & 31;
  int r0, r1;
  if (bundles) {
    r0 = __ldg(bundles + b);
    r1 = __ldg(bundles + b + 1);
  } else {
    r0 = b * 32;
    r1 = min(r0 + 32, n);
  }
  const int j0 = __ldg(ia + r0), j1 = __ldg(ia + r1);
  if (j1 - j0 > kBundleNnz) {
    for (int r = r0; r < r1; ++r) {
      const int k0 = __ldg(ia + r), k1 = __ldg(ia + r + 1);
      T s = T(0);
      for (int j = k0 + lane; j < k1; j += 32) {
        const T xv = xf(__ldg(ja + j));
        s = EXACT ? add_rn(s, mul_rn(mul_rn(alpha, __ldg(a + j)), xv)) : fma_rn(__ldg(a + j), xv, s);
      }
      s = warp_sum(s);
      if (lane == 0) ep.store(r, add_rn(ep.init(r), s));
    }
    __syncwarp();
    return;
  }
  // staging, 4 entries per lane in flight: all index/value loads of a group
  // are issued before its x gathers, which are issued before any use
  const int cnt = j1 - j0;
  for (int e0 = 0; e0 < cnt; e0 += 128) {
    int c[4];
    T av[4], xv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * 32 + lane;
      c[u] = e < cnt ? __ldg(ja + j0 + e) : -1;
      if (EXACT) av[u] = e < cnt ? __ldg(a + j0 + e) : T(0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) xv[u] = c[u] >= 0 ? xf(c[u]) : T(0);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * 32 + lane;
      if (e < cnt) stage[e] = EXACT ? mul_rn(mul_rn(alpha, av[u]), xv[u]) : xv[u];
    }
  }
  __syncwarp();
  const int r = r0 + lane;
  if (r < r1) {
    const int e0 = __ldg(ia + r) - j0, e1 = __ldg(ia + r + 1) - j0;
    T acc = ep.init(r);
    if (EXACT) {
      for (int e = e0; e < e1; ++e) acc = add_rn(acc, stage[e]);
    } else {
      for (int e = e0; e < e1; ++e) acc = fma_rn(__ldg(a + j0 + e), stage[e], acc);
    }
    ep.store(r, acc);
  }
  __syncwarp();
}

// Simple x functor: x[col].
template <typename T>
struct XPlain {
  const T* __restrict__ x;
  __device__ __forceinline__ T operator()(int c) const { return __ldg(x + c); }
};

}  // namespace gb
