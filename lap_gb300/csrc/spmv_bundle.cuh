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
//   void prefetch(int row)    -> optional: issue the loads store() will need
//                                (called at the start of the row's bundle)
// X contract:
//   T operator()(int col)     -> x value at col
template <typename EP>
__device__ __forceinline__ auto ep_prefetch(EP& ep, int r, int) -> decltype(ep.prefetch(r), void()) {
  ep.prefetch(r);
}
template <typename EP>
__device__ __forceinline__ void ep_prefetch(EP&, int, long) {}

// Values of a row held in registers from the start of its bundle (FMA
// form): a stencil row's whole dependency list is in flight at once.
constexpr int kSpmvHeld = 8;
// 1: bundles whose rows all have at most kSpmvHeld entries take the
// per-lane form (no staging).
#ifndef GB_SPMV_SHORT_ROWS
#define GB_SPMV_SHORT_ROWS 1
#endif
// 1: the FMA form stages the matrix values beside the gathered x (coalesced
// loads; the row sums then read shared memory only), in bundles of half the
// entries so the staging takes the same shared memory.
#ifndef GB_SPMV_STAGE_A
#define GB_SPMV_STAGE_A 0
#endif

// bundles == nullptr selects the plan-free layout: bundle b is rows
// [32b, 32b+32); one whose entries overflow the staging buffer is walked row
// by row with the whole warp.
//
// Latency structure of a bundle: its row bounds (one coalesced load per
// lane) -> the column indices (coalesced over the bundle's entries) and, in
// the FMA form, the row's first kSpmvHeld values -> the x gathers -> the row
// sums.  The epilogue's loads are issued before the row bounds.
// The head of bundle b: its rows [r0, r1) and this lane's row bounds
// [rs, re) -- the loads a bundle's chain starts with.  The grid-stride loops
// load the next bundle's head before they work on the current one
// (spmv_bundles), so that round trip overlaps the bundle in hand.
struct BundleHead {
  int r0, r1, rs, re;
};
__device__ __forceinline__ BundleHead bundle_head(int b, int n, const int* __restrict__ bundles,
                                                  const int* __restrict__ ia) {
  BundleHead h;
  if (bundles) {
    h.r0 = __ldg(bundles + b);
    h.r1 = __ldg(bundles + b + 1);
  } else {
    h.r0 = b * 32;
    h.r1 = min(h.r0 + 32, n);
  }
  const int lane = threadIdx.x & 31;
  const bool own = lane < h.r1 - h.r0;
  h.rs = own ? __ldg(ia + h.r0 + lane) : 0;
  h.re = own ? __ldg(ia + h.r0 + lane + 1) : 0;
  return h;
}

template <typename T, bool EXACT, typename XF, typename EP>
__device__ __forceinline__ void spmv_bundle_h(const BundleHead& h, const int* __restrict__ ia,
                                              const int* __restrict__ ja, const T* __restrict__ a, T alpha, XF& xf,
                                              EP& ep, T* stage) {
  const int lane = threadIdx.x & 31;
  const int r0 = h.r0, r1 = h.r1;
  const int nr = r1 - r0;
  const int r = r0 + lane;
  const bool own = lane < nr;
  // the epilogue's loads first: they do not depend on the row bounds (a
  // row of the long-row path below issues them again, in lane 0)
  if (own) ep_prefetch(ep, r, 0);
  // this lane's row bounds; lane nr-1's end is the bundle's
  const int rs = h.rs;
  const int re = h.re;
  const int j0 = __shfl_sync(0xffffffffu, rs, 0);
  const int j1 = __shfl_sync(0xffffffffu, re, nr - 1);
  if (j1 - j0 > (GB_SPMV_STAGE_A && !EXACT ? kBundleNnz / 2 : kBundleNnz)) {
    for (int rr = r0; rr < r1; ++rr) {
      const int k0 = __ldg(ia + rr), k1 = __ldg(ia + rr + 1);
      T s = T(0);
      for (int j = k0 + lane; j < k1; j += 32) {
        const T xv = xf(__ldg(ja + j));
        s = EXACT ? add_rn(s, mul_rn(mul_rn(alpha, __ldg(a + j)), xv)) : fma_rn(__ldg(a + j), xv, s);
      }
      s = warp_sum(s);
      if (lane == 0) {
        ep_prefetch(ep, rr, 0);
        ep.store(rr, add_rn(ep.init(rr), s));
      }
    }
    __syncwarp();
    return;
  }
#if GB_SPMV_SHORT_ROWS
  // Every row of the bundle has at most kSpmvHeld entries (stencils): each
  // lane loads its own row's columns and values and gathers its x values,
  // all of them in flight at once -- no staging pass.  The same FMA chain,
  // in the same order, as the staged form below.
  if (!EXACT && __all_sync(0xffffffffu, !own || re - rs <= kSpmvHeld)) {
    if (own) {
      T acc = ep.init(r);
      int c[kSpmvHeld];
      T av[kSpmvHeld], xv[kSpmvHeld];
#pragma unroll
      for (int u = 0; u < kSpmvHeld; ++u) {
        const bool in = rs + u < re;
        c[u] = in ? __ldg(ja + rs + u) : -1;
        av[u] = in ? __ldg(a + rs + u) : T(0);
      }
#pragma unroll
      for (int u = 0; u < kSpmvHeld; ++u) xv[u] = c[u] >= 0 ? xf(c[u]) : T(0);
#pragma unroll
      for (int u = 0; u < kSpmvHeld; ++u)
        if (c[u] >= 0) acc = fma_rn(av[u], xv[u], acc);
      ep.store(r, acc);
    }
    __syncwarp();
    return;
  }
#endif
  T acc = T(0);
  T held[kSpmvHeld];
  if (own) {
    acc = ep.init(r);
    if (!EXACT && !GB_SPMV_STAGE_A) {
#pragma unroll
      for (int u = 0; u < kSpmvHeld; ++u) held[u] = rs + u < re ? __ldg(a + rs + u) : T(0);
    }
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
      if (EXACT || GB_SPMV_STAGE_A) av[u] = e < cnt ? __ldg(a + j0 + e) : T(0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) xv[u] = c[u] >= 0 ? xf(c[u]) : T(0);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = e0 + u * 32 + lane;
      if (e < cnt) stage[e] = EXACT ? mul_rn(mul_rn(alpha, av[u]), xv[u]) : xv[u];
      if (!EXACT && GB_SPMV_STAGE_A && e < cnt) stage[kBundleNnz / 2 + e] = av[u];
    }
  }
  __syncwarp();
  if (own) {
    const int e0 = rs - j0, e1 = re - j0;
    if (EXACT) {
      for (int e = e0; e < e1; ++e) acc = add_rn(acc, stage[e]);
    } else if (GB_SPMV_STAGE_A) {
      for (int e = e0; e < e1; ++e) acc = fma_rn(stage[kBundleNnz / 2 + e], stage[e], acc);
    } else {
#pragma unroll
      for (int u = 0; u < kSpmvHeld; ++u)
        if (e0 + u < e1) acc = fma_rn(held[u], stage[e0 + u], acc);
      for (int e = e0 + kSpmvHeld; e < e1; ++e) acc = fma_rn(__ldg(a + j0 + e), stage[e], acc);
    }
    ep.store(r, acc);
  }
  __syncwarp();
}

template <typename T, bool EXACT, typename XF, typename EP>
__device__ __forceinline__ void spmv_bundle(int b, int n, const int* __restrict__ bundles,
                                            const int* __restrict__ ia, const int* __restrict__ ja,
                                            const T* __restrict__ a, T alpha, XF& xf, EP& ep, T* stage) {
  spmv_bundle_h<T, EXACT>(bundle_head(b, n, bundles, ia), ia, ja, a, alpha, xf, ep, stage);
}

// Bundles b0, b0 + step, ... < nb, each bundle's head loaded while the one
// before it is worked on.
template <typename T, bool EXACT, typename XF, typename EP>
__device__ __forceinline__ void spmv_bundles(int b0, int step, int nb, int n, const int* __restrict__ bundles,
                                             const int* __restrict__ ia, const int* __restrict__ ja,
                                             const T* __restrict__ a, T alpha, XF& xf, EP& ep, T* stage) {
  if (b0 >= nb) return;
  BundleHead h = bundle_head(b0, n, bundles, ia);
  for (int b = b0; b < nb; b += step) {
    const int bn = b + step;
    const BundleHead hn = bn < nb ? bundle_head(bn, n, bundles, ia) : h;
    spmv_bundle_h<T, EXACT>(h, ia, ja, a, alpha, xf, ep, stage);
    h = hn;
  }
}

// Simple x functor: x[col].
template <typename T>
struct XPlain {
  const T* __restrict__ x;
  __device__ __forceinline__ T operator()(int c) const { return __ldg(x + c); }
};

}  // namespace gb
