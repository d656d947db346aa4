// pcg.cu -- the device-resident PCG of cg.c:5-140 with fused kernels.
//
// Per iteration LAP's CUDA build launches ~9 library kernels and reads three
// dot products back to the host (cg.c:73,90,102).  Here one iteration is:
//
//   Jacobi / none : [spmv_pq] [update]                      2 kernels
//   ichol, GS_std : [spmv_pq] [lower solve + update] [upper solve + r'w]
//   others        : [spmv_pq] [update] [LAP preconditioner kernels] [r'w]
//
//   spmv_pq  s = A w; q = s + beta*q_old; p = w + beta*p_old (cg.c:81-85 by
//            linearity: A(w + beta p) = A w + beta A p), p'q reduced.  The
//            SpMV gathers only w and spends one FMA per nonzero -- GB300's
//            FP64 rate is 1/64 of FP32, so FP64 instructions, not bytes,
//            bound a naive fused form;
//   update   x += alpha p, r -= alpha q, w = D^-1 r (Jacobi), r'r and r'w
//            reduced, cg.c's stopping rule applied by the last block.
//
// All scalars (rho, p'q, alpha, beta, the residual history) stay in device
// memory (PcgState); the loop runs as a CUDA-graph while node whose
// condition the checking kernel sets, so a whole solve is one graph launch.
// Reductions are deterministic (fixed partial slots summed in order).
#include <algorithm>
#include <cstring>

#include "gb_common.cuh"
#include "kernels.h"
#include "pcg.h"
#include "pcg_state.cuh"
#include "sptrsv.h"
#include "system.h"

namespace gb {

constexpr int kThreads = 256;
// grid-stride elements per step in the elementwise kernels (128^3 update:
// 33.8 us at 1, 28.4 at 4, 39.7 at 8 -- registers then halve the resident
// blocks; a grid of twice the blocks measured 36.6)
constexpr int kEwUnroll = 4;

template <typename T>
struct VecPtrs {
  T *x, *r, *w, *p0, *p1, *q, *t, *s;
};

// Last-block reduction helper: block sums NV values, publishes, and the last
// block (block-uniform result) sums all partials.  Ticket reset by the last.
template <int NV>
__device__ __forceinline__ bool reduce_last(double (&v)[NV], double* part, int nblocks, int slot,
                                            unsigned* ticket, double* sm) {
  block_sum<NV>(v, sm);
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) part[k * nblocks + slot] = v[k];
    __threadfence();
    last = atomicAdd(ticket, 1u) == (unsigned)nblocks - 1u;
    if (last) {
      *ticket = 0u;
      __threadfence();
    }
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();  // acquire side: the other blocks' partials, read by every thread below
  double t[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    t[k] = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) t[k] += ld_relaxed(part + k * nblocks + i);
  }
  block_sum<NV>(t, sm);
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = t[k];
  return true;  // result valid in thread 0
}

// ------------------------------------------------------------ prologue
// r = b - A x (x_zero: r = b), w = D^-1 r for Jacobi, r'r and (Jacobi/none)
// rho = r'w; fills the lower solve's output t with the sentinel.
template <typename T, int WK>
__global__ void __launch_bounds__(kThreads)
    resid_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                 const int* __restrict__ ja, const T* __restrict__ a, const T* b,
                 const T* __restrict__ x, int x_zero, T* r, T* w, const T* __restrict__ d_r,
                 T* tfill, PcgState* st, double* part, double* hist) {
  __shared__ T stage[kThreads / 32][kBundleNnz];
  __shared__ double sm[2 * kThreads / 32];
  const int wid = threadIdx.x >> 5;
  struct Ep {
    const T* b;
    T *r, *w;
    const T* d_r;
    T* tf;
    double a0, a1;
    __device__ T init(int) const { return T(0); }
    __device__ void store(int i, T v) {
      const T ri = sub_rn(b[i], v);
      r[i] = ri;
      a0 += (double)ri * (double)ri;
      if (WK == WK_JACOBI) {
        const T wi = d_r[i] * ri;
        w[i] = wi;
        a1 += (double)ri * (double)wi;
      }
      if (tf) tf[i] = sentinel<T>();
    }
  } ep{b, r, w, d_r, tfill, 0.0, 0.0};
  if (x_zero) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) ep.store(i, T(0));
  } else {
    XPlain<T> xf{x};
    for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
      spmv_bundle<T, false>(bb, n, bundles, ia, ja, a, T(1), xf, ep, stage[wid]);
  }
  double acc[2] = {ep.a0, ep.a1};
  if (reduce_last<2>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_RESID], sm) && threadIdx.x == 0) {
    const double res0 = sqrt(acc[0]);
    st->res0 = res0;
    st->rr = acc[0];
    st->tolrel = st->spare0 * res0;  // spare0 carries tol
    if (st->hist_len > 0) hist[0] = res0;
    if (WK == WK_NONE) st->rho = acc[0];
    if (WK == WK_JACOBI) st->rho = acc[1];
    st->rho_prev = 0.0;
  }
}

// ------------------------------------------------------------ spmv_pq
// Five resident blocks per SM, as spmv_pq_split_kernel: the FP64 form then
// holds 48 registers with a 72-byte spill instead of 64 (128^3: 69.0 ->
// 62.4 us); the FP32 form needs 48 either way.
template <typename T, int WK>
__global__ void __launch_bounds__(kThreads, 5)
    spmv_pq_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                   const int* __restrict__ ja, const T* __restrict__ a, const T* __restrict__ w,
                   T* p, T* q, T* tfill, PcgState* st, double* part,
                   cudaGraphConditionalHandle cond, int has_cond) {
  __shared__ T stage[kThreads / 32][kBundleNnz];
  __shared__ double sm[kThreads / 32];
  // Loop guard, independent of the checking kernel later in the body: a
  // graph while loop can never run more than maxit + 8 bodies.
  if (has_cond && blockIdx.x == 0 && threadIdx.x == 0) {
    const int g = ++st->spare_guard;
    if (g > st->maxit + 8) set_cond(cond, true, false);
  }
  if (st->done) return;  // uniform across the grid
  const bool first = st->iter == 0;
  const T beta = first ? T(0) : (T)(st->rho / st->rho_prev);
  XPlain<T> xf{w};
  struct Ep {
    const T* w;
    T *p, *q, *tf;
    T beta;
    bool first;
    double pq;
    T wi, po, qo;  // loaded with the row bounds (prefetch)
    __device__ void prefetch(int i) {
      wi = w[i];
      po = first ? T(0) : p[i];
      qo = first ? T(0) : q[i];
    }
    __device__ T init(int) const { return T(0); }
    __device__ void store(int i, T s) {
      const T pi = first ? wi : fma_rn(beta, po, wi);
      const T qi = first ? s : fma_rn(beta, qo, s);
      p[i] = pi;
      q[i] = qi;
      pq += (double)pi * (double)qi;
      if (tf) tf[i] = sentinel<T>();
    }
  } ep{w, p, q, tfill, beta, first, 0.0, T(0), T(0), T(0)};
  const int wid = threadIdx.x >> 5;
  for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
    spmv_bundle<T, false>(bb, n, bundles, ia, ja, a, T(1), xf, ep, stage[wid]);
  double acc[1] = {ep.pq};
  if (reduce_last<1>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_PQ], sm) && threadIdx.x == 0)
    st->pq = acc[0];
}

// ------------------------------------------------------------ update
template <typename T, int WK>
__global__ void __launch_bounds__(kThreads)
    update_kernel(int n, T* __restrict__ x, T* __restrict__ r, T* __restrict__ w, const T* __restrict__ p,
                  const T* __restrict__ q,
                  const T* __restrict__ d_r, PcgState* st, double* part, double* hist,
                  cudaGraphConditionalHandle cond, int has_cond) {
  __shared__ double sm[2 * kThreads / 32];
  if (st->done) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_cond(cond, has_cond, false);
    return;
  }
  double alpha;
  if (!pcg_alpha(st, &alpha)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->done = 1;
      st->flag = 2;
      st->status = GB_BREAKDOWN;
      set_cond(cond, has_cond, false);
    }
    return;
  }
  const T al = (T)alpha, nal = (T)(-alpha);
  double acc[2] = {0.0, 0.0};
  auto one = [&](int i, T pv, T xv, T qv, T rv, T dv) {
    x[i] = fma_rn(al, pv, xv);
    const T ri = fma_rn(nal, qv, rv);
    r[i] = ri;
    acc[0] += (double)ri * (double)ri;
    if (WK == WK_JACOBI) {
      const T wi = dv * ri;
      w[i] = wi;
      acc[1] += (double)ri * (double)wi;
    }
  };
  // kEwUnroll grid-stride elements per step, all their loads issued first:
  // a thread keeps kEwUnroll x 4-5 loads in flight instead of 4-5
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + (kEwUnroll - 1) * stride < n; i += kEwUnroll * stride) {
    T pv[kEwUnroll], xv[kEwUnroll], qv[kEwUnroll], rv[kEwUnroll], dv[kEwUnroll];
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) {
      const int j = i + u * stride;
      pv[u] = p[j];
      xv[u] = x[j];
      qv[u] = q[j];
      rv[u] = r[j];
      dv[u] = WK == WK_JACOBI ? d_r[j] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) one(i + u * stride, pv[u], xv[u], qv[u], rv[u], dv[u]);
  }
  for (; i < n; i += stride) one(i, p[i], x[i], q[i], r[i], WK == WK_JACOBI ? d_r[i] : T(0));
  if (reduce_last<2>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_UPD], sm) && threadIdx.x == 0) {
    pcg_check(st, acc[0], hist);
    if (WK != WK_PREC) {
      st->rho_prev = st->rho;
      st->rho = WK == WK_NONE ? acc[0] : acc[1];
    }
    set_cond(cond, has_cond, !st->done && st->body_count++ < st->maxit + 4);
  }
}

// rho = r'w after a composed preconditioner (PREC kind), and after the
// split recurrence's FP32 upper solve (FP64 r, FP32 w): rho_prev <- rho.
template <typename T, typename TW = T>
__global__ void __launch_bounds__(kThreads)
    rho_kernel(int n, const T* __restrict__ r, const TW* __restrict__ w, PcgState* st,
               double* part) {
  __shared__ double sm[kThreads / 32];
  if (st->done) return;
  double acc[1] = {0.0};
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + (kEwUnroll - 1) * stride < n; i += kEwUnroll * stride) {
    T rv[kEwUnroll];
    TW wv[kEwUnroll];
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) {
      rv[u] = r[i + u * stride];
      wv[u] = w[i + u * stride];
    }
#pragma unroll
    for (int u = 0; u < kEwUnroll; ++u) acc[0] = fma((double)rv[u], (double)wv[u], acc[0]);
  }
  for (; i < n; i += stride) acc[0] = fma((double)r[i], (double)w[i], acc[0]);
  if (reduce_last<1>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_RHO], sm) && threadIdx.x == 0) {
    st->rho_prev = st->rho;
    st->rho = acc[0];
  }
}

// ------------------------------------------------------------ tri ops
// The PCG's triangular solves carry no FP64 vector work (GB300 issues FP64
// at 1/64 of the FP32 rate, and anything queued on that pipe sits in front
// of the solve's dependency chain): the x / r update runs before the lower
// solve (update_kernel), r'w after the upper (rho_kernel), and GS_std's
// right-hand side r - A t before its backward sweep (gs_rhs_kernel).
// Measured on the 128^3 split solve: r'w fused into the FP32 upper solve's
// epilogue (r_i loaded with the record, one FP64 FMA per row, per-tile sums)
// took the solve from 337 to 389-397 us, against 18 us for rho_kernel.

// Lower solve: the residual r is the right-hand side (rounded to the solve's
// type in the split recurrence); also pre-fills the upper solve's output.
template <typename T, typename TR>
struct OpSplitLower {
  static constexpr bool kPollValues = true;
  const TR* r;
  T* sfill;
  PcgState* st;
  bool dn;
  __device__ void begin() { dn = st->done != 0; }
  __device__ bool active() const { return !dn; }
  __device__ void inactive_end() {}
  struct Pre {
    TR r;
  };
  struct DPre {};
  __device__ Pre pre(int i) const { return {r[i]}; }
  __device__ T rhs(int, const Pre& v) const { return (T)v.r; }
  __device__ DPre dpre(int) const { return {}; }
  __device__ void done(int i, T, const DPre&) {
    if (sfill) sfill[i] = sentinel<T>();
  }
  __device__ void prefetch(int r0, int r1, int part) const {
    prefetch_rows_l2(r, r0, r1, part, kTriProdLanes);
  }
  __device__ void chunk_end(int, int nchunks, unsigned* ticket, double*) {
    if (threadIdx.x == 0) chunk_finished(ticket, nchunks);
  }
};

// IC(0) upper solve: y = U^{-1} t only; r'w follows in rho_kernel.
template <typename T>
struct OpSplitUpper {
  // FP32 upper solves poll values (one loop over a lane's pending ones),
  // on plane tiles in pushing clusters like the lower: 128^3 upper 267 ->
  // 250 us.  On two-plane tiles in pulling clusters polling changed
  // nothing, and FP64 upper solves measured slower polling.
  static constexpr bool kPollValues = sizeof(T) == 4;
  const T* t;
  PcgState* st;
  bool dn;
  __device__ void begin() { dn = st->done != 0; }
  __device__ bool active() const { return !dn; }
  __device__ void inactive_end() {}
  struct Pre {
    T t;
  };
  struct DPre {};
  __device__ Pre pre(int i) const { return {t[i]}; }
  __device__ T rhs(int, const Pre& v) const { return v.t; }
  __device__ DPre dpre(int) const { return {}; }
  __device__ void done(int, T, const DPre&) {}
  __device__ void prefetch(int r0, int r1, int part) const {
    prefetch_rows_l2(t, r0, r1, part, kTriProdLanes);
  }
  __device__ void chunk_end(int, int nchunks, unsigned* ticket, double*) {
    if (threadIdx.x == 0) chunk_finished(ticket, nchunks);
  }
};

// GS_std (k = 1) backward sweep, with its right-hand side g = r - A t
// computed beforehand by gs_rhs_kernel: y = (D+U)^{-1} g, w = t + y
// (GS.c:34-40); r'w follows in rho_kernel.
template <typename T>
struct OpSplitGsUpper {
  // FP32 sweeps poll values, as OpSplitUpper<float> (128^3 GS_std split
  // PCG: backward sweep with g and r'w 327 -> 310 us, 148.4 -> 144.0 ms)
  static constexpr bool kPollValues = sizeof(T) == 4;
  const T* g;
  const T* t;
  T* w;
  PcgState* st;
  bool dn;
  __device__ void begin() { dn = st->done != 0; }
  __device__ bool active() const { return !dn; }
  __device__ void inactive_end() {}
  struct Pre {
    T g;
  };
  struct DPre {
    T t;
  };
  __device__ Pre pre(int i) const { return {g[i]}; }
  __device__ T rhs(int, const Pre& v) const { return v.g; }
  __device__ DPre dpre(int i) const { return {t[i]}; }
  __device__ void done(int i, T y, const DPre& v) { w[i] = v.t + y; }
  __device__ void prefetch(int r0, int r1, int part) const {
    prefetch_rows_l2(g, r0, r1, part, kTriProdLanes);
    prefetch_rows_l2(t, r0, r1, part, kTriProdLanes);
  }
  __device__ void chunk_end(int, int nchunks, unsigned* ticket, double*) {
    if (threadIdx.x == 0) chunk_finished(ticket, nchunks);
  }
};

// g = r - A t (GS.c:34-35) in the solve's type T, as a bandwidth pass over
// A before the backward sweep: acc = r; acc = fma(-a_ij, t_j, acc) along
// the row.  fma(-a, t, acc) = -fma(a, t, -acc) exactly, so the row-bundle
// SpMV computes that chain negated, starting from -r (rows of more than
// kBundleNnz entries are summed by the whole warp instead).
template <typename T, typename TR>
__global__ void __launch_bounds__(kThreads)
    gs_rhs_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                  const int* __restrict__ ja, const T* __restrict__ a, const T* __restrict__ t,
                  const TR* __restrict__ r, T* g, const PcgState* st) {
  __shared__ T stage[kThreads / 32][kBundleNnz];
  if (st->done) return;
  XPlain<T> xf{t};
  struct Ep {
    const TR* r;
    T* g;
    __device__ T init(int i) const { return -(T)r[i]; }
    __device__ void store(int i, T v) { g[i] = -v; }
  } ep{r, g};
  const int wid = threadIdx.x >> 5;
  for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
    spmv_bundle<T, false>(bb, n, bundles, ia, ja, a, T(1), xf, ep, stage[wid]);
}

// ------------------------------------------------------------ spmv_pq (split)
// Split precision: q = A w + beta q and p = w + beta p with w the FP32 output
// of the preconditioner, A's FP32 values and FP32 products (A w), and p, q,
// beta and p'q in FP64.  By linearity q = A p as in spmv_pq_kernel.
// Five resident blocks per SM (at most 51 registers, no spills; 64 without
// the bound): this latency-bound kernel needs the warps (128^3: 48.3 ->
// 45.6 us; six or eight blocks spill and measured 48.1 / 53.1 us).
__global__ void __launch_bounds__(kThreads, 5)
    spmv_pq_split_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                         const int* __restrict__ ja, const float* __restrict__ a,
                         const float* __restrict__ w, double* p, double* q, float* tfill,
                         PcgState* st, double* part, cudaGraphConditionalHandle cond, int has_cond) {
  __shared__ float stage[kThreads / 32][kBundleNnz];
  __shared__ double sm[kThreads / 32];
  if (has_cond && blockIdx.x == 0 && threadIdx.x == 0) {
    const int g = ++st->spare_guard;
    if (g > st->maxit + 8) set_cond(cond, true, false);
  }
  if (st->done) return;  // uniform across the grid
  const bool first = st->iter == 0;
  const double beta = first ? 0.0 : st->rho / st->rho_prev;
  XPlain<float> xf{w};
  struct Ep {
    const float* w;
    double *p, *q;
    float* tf;
    double beta;
    bool first;
    double pq;
    float wi;
    double po, qo;  // loaded with the row bounds (prefetch)
    __device__ void prefetch(int i) {
      wi = w[i];
      po = first ? 0.0 : p[i];
      qo = first ? 0.0 : q[i];
    }
    __device__ float init(int) const { return 0.0f; }
    __device__ void store(int i, float s) {
      const double pi = first ? (double)wi : fma_rn(beta, po, (double)wi);
      const double qi = first ? (double)s : fma_rn(beta, qo, (double)s);
      p[i] = pi;
      q[i] = qi;
      pq = fma_rn(pi, qi, pq);
      if (tf) tf[i] = sentinel<float>();
    }
  } ep{w, p, q, tfill, beta, first, 0.0, 0.0f, 0.0, 0.0};
  const int wid = threadIdx.x >> 5;
  // each bundle's head loaded while the previous bundle is worked on (128^3:
  // 45.9 -> 44.7 us; the FP64 kernel, which then spills more, measured
  // slower with it: 62.1 -> 68 us)
  spmv_bundles<float, false>(blockIdx.x * (kThreads / 32) + wid, gridDim.x * (kThreads / 32), nb, n, bundles, ia, ja,
                             a, 1.0f, xf, ep, stage[wid]);
  double acc[1] = {ep.pq};
  if (reduce_last<1>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_PQ], sm) && threadIdx.x == 0)
    st->pq = acc[0];
}

// ------------------------------------------------------------ true residual
// ||b - A x|| and ||b|| in FP64 after the solve (cg.c:113-117).
__global__ void __launch_bounds__(kThreads)
    true_resid_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                      const int* __restrict__ ja, const double* __restrict__ a,
                      const double* __restrict__ b, const double* __restrict__ x, double* out2,
                      PcgState* st, double* part) {
  __shared__ double stage[kThreads / 32][kBundleNnz];
  __shared__ double sm[2 * kThreads / 32];
  struct Ep {
    const double* b;
    double a0, a1;
    __device__ double init(int) const { return 0.0; }
    __device__ void store(int i, double v) {
      const double ri = b[i] - v;
      a0 += ri * ri;
      a1 += b[i] * b[i];
    }
  } ep{b, 0.0, 0.0};
  XPlain<double> xf{x};
  const int wid = threadIdx.x >> 5;
  for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
    spmv_bundle<double, false>(bb, n, bundles, ia, ja, a, 1.0, xf, ep, stage[wid]);
  double acc[2] = {ep.a0, ep.a1};
  if (reduce_last<2>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_TRUE], sm) && threadIdx.x == 0) {
    out2[0] = sqrt(acc[0]);
    out2[1] = sqrt(acc[1]);
  }
}

// ------------------------------------------------------------ mixed precision helpers
// Outer FP64 residual r = b - A x, its norm, stored as the inner recurrence's
// residual (FP32 for the FP32 recurrence, FP64 for the split one; x32, when
// given, is the FP32 correction to clear), and the refinement stopping test
// against tol * ||b - A x0||.
template <typename TR>
__global__ void __launch_bounds__(kThreads)
    outer_resid_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                       const int* __restrict__ ja, const double* __restrict__ a,
                       const double* __restrict__ b, const double* __restrict__ x, TR* r32,
                       float* x32, PcgState* so, double* part, int first) {
  __shared__ double stage[kThreads / 32][kBundleNnz];
  __shared__ double sm[kThreads / 32];
  struct Ep {
    const double* b;
    TR* r32;
    float* x32;
    double a0;
    __device__ double init(int) const { return 0.0; }
    __device__ void store(int i, double v) {
      const double ri = b[i] - v;
      r32[i] = (TR)ri;
      if (x32) x32[i] = 0.0f;
      a0 += ri * ri;
    }
  } ep{b, r32, x32, 0.0};
  XPlain<double> xf{x};
  const int wid = threadIdx.x >> 5;
  for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
    spmv_bundle<double, false>(bb, n, bundles, ia, ja, a, 1.0, xf, ep, stage[wid]);
  double acc[1] = {ep.a0};
  if (reduce_last<1>(acc, part, gridDim.x, blockIdx.x, &so->tk[TK_RESID], sm) && threadIdx.x == 0) {
    const double res = sqrt(acc[0]);
    if (first) {
      so->res0 = res;
      so->tolrel = so->spare0 * res;
    }
    so->rr = acc[0];
    if (!(res == res)) {
      so->done = 1;
      so->flag = 2;
      so->status = GB_BREAKDOWN;
    } else if (res < so->tolrel) {
      so->done = 1;
      so->flag = 0;
      so->status = GB_OK;
    }
  }
}

__global__ void add_correction_kernel(int n, double* x, const float* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] += (double)d[i];
}

// Residual replacement (mixed precision): after r was replaced by the FP64
// true residual, the paused recurrence resumes -- p, q, rho_prev and the
// iteration count are kept; the pause threshold moves to delta*||r||, but not
// below the solve's own target, so the last cycle stops at the tolerance.
__global__ void resume_kernel(PcgState* st, const PcgState* so, double delta) {
  st->done = 0;
  st->flag = 1;
  st->status = GB_OK;
  st->spare_guard = 0;
  st->body_count = 0;
  st->tolrel = fmax(delta * sqrt(so->rr), so->tolrel);
}

// Jacobi / none after a residual replacement: w = D^-1 r, rho rolled.
template <typename T, int WK>
__global__ void __launch_bounds__(kThreads)
    refresh_kernel(int n, const T* __restrict__ r, T* w, const T* __restrict__ d_r, PcgState* st,
                   double* part) {
  __shared__ double sm[kThreads / 32];
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T ri = r[i];
    if (WK == WK_JACOBI) {
      const T wi = d_r[i] * ri;
      w[i] = wi;
      acc[0] += (double)ri * (double)wi;
    } else {
      acc[0] += (double)ri * (double)ri;
    }
  }
  if (reduce_last<1>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_RHO], sm) && threadIdx.x == 0) {
    st->rho_prev = st->rho;
    st->rho = acc[0];
  }
}

// ================================================================ host side
// One full wave of the bundle kernels (their occupancy is set by the staging
// buffer, kThreads/32 x kBundleNnz x sizeof(T)).
template <typename T>
static int grid_for_bundles(int nb) {
  return wave_grid(spmv_pq_kernel<T, WK_PREC>, kThreads, ceil_div(nb, kThreads / 32));
}
static int grid_ew(int n) { return std::max(1, std::min(ceil_div(n, kThreads), reduction_grid())); }

template <typename T>
static VecPtrs<T> vecs(gb_system sys);
template <>
VecPtrs<double> vecs<double>(gb_system sys) {
  auto& v = sys->v64;
  return {v.x, v.r, v.w, v.p0, v.p1, v.q, v.t, v.s};
}
template <>
VecPtrs<float> vecs<float>(gb_system sys) {
  auto& v = sys->v32;
  return {v.x, v.r, v.w, v.p0, v.p1, v.q, v.t, v.s};
}
template <typename T>
static const T* mat_vals(gb_system sys);
template <>
const double* mat_vals<double>(gb_system sys) { return sys->a; }
template <>
const float* mat_vals<float>(gb_system sys) { return sys->a32; }
template <typename T>
static const T* dr_vals(gb_system sys);
template <>
const double* dr_vals<double>(gb_system sys) { return sys->d_r; }
template <>
const float* dr_vals<float>(gb_system sys) { return sys->d_r32; }

int prec_wkind(int prec, int k) {
  if (prec == GB_PREC_NONE) return WK_NONE;
  if (prec == GB_PREC_LINE_JACOBI) return WK_JACOBI;
  (void)k;
  return WK_PREC;
}
bool prec_fused_tri(int prec, int k) {
  return prec == GB_PREC_ICHOL || (prec == GB_PREC_GS_STD && k == 1);
}

// The lower solve; with do_update, preceded by the x / r update and the
// stopping test (update_kernel, which also ends the graph's loop).
template <typename T>
static int launch_lower(gb_system sys, PcgState* st, int do_update, cudaGraphConditionalHandle cond,
                        int has_cond) {
  auto v = vecs<T>(sys);
  if (do_update) {
    update_kernel<T, WK_PREC><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(
        sys->n, v.x, v.r, nullptr, v.p0, v.q, nullptr, st, sys->part, sys->hist, cond, has_cond);
    GB_CUDA_TRY(cudaGetLastError());
  }
  const TriPlan& L = sizeof(T) == 8 ? sys->L : sys->L32;
  OpSplitLower<T, T> op{v.r, v.s, st, false};
  return tri_launch<T, OpSplitLower<T, T>, false>(L, tri_args<T>(L, v.t, sys->err, true), op, sys->s);
}

// The upper solve and r'w (GS_std: g = r - A t first; p1 holds g).
template <typename T>
static int launch_upper(gb_system sys, PcgState* st) {
  auto v = vecs<T>(sys);
  const TriPlan& U = sizeof(T) == 8 ? sys->U : sys->U32;
  if (sys->prec == GB_PREC_ICHOL) {
    OpSplitUpper<T> op{v.t, st, false};
    GB_TRY((tri_launch<T, OpSplitUpper<T>, false>(U, tri_args<T>(U, v.s, sys->err, true), op, sys->s)));
    rho_kernel<T><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(sys->n, v.r, v.s, st, sys->part);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  const int nb = sys->plan.nbundles;
  gs_rhs_kernel<T, T><<<wave_grid(gs_rhs_kernel<T, T>, kThreads, ceil_div(nb, kThreads / 32)), kThreads, 0,
                        sys->s>>>(sys->n, nb, sys->plan.bundles, sys->ia, sys->ja, mat_vals<T>(sys), v.t, v.r,
                                  v.p1, st);
  GB_CUDA_TRY(cudaGetLastError());
  OpSplitGsUpper<T> op{v.p1, v.t, v.w, st, false};
  GB_TRY((tri_launch<T, OpSplitGsUpper<T>, false>(U, tri_args<T>(U, v.s, sys->err, true), op, sys->s)));
  rho_kernel<T><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(sys->n, v.r, v.w, st, sys->part);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// w buffer the spmv_pq kernel gathers: ichol's w is the upper solve's output
// s; none uses r itself; the rest write w.
template <typename T>
static const T* w_buffer(gb_system sys) {
  auto v = vecs<T>(sys);
  if (sys->prec == GB_PREC_ICHOL) return v.s;
  if (sys->prec == GB_PREC_NONE) return v.r;
  return v.w;
}

template <typename T>
int launch_prologue(gb_system sys, PcgState* st, int x_zero, const T* b) {
  auto v = vecs<T>(sys);
  const int wk = prec_wkind(sys->prec, sys->k);
  const bool tri = prec_fused_tri(sys->prec, sys->k);
  const int nb = sys->plan.nbundles;
  const int g = grid_for_bundles<T>(nb);
  const T* a = mat_vals<T>(sys);
  const T* dr = dr_vals<T>(sys);
#define GB_RESID(WKV)                                                                          \
  resid_kernel<T, WKV><<<g, kThreads, 0, sys->s>>>(sys->n, nb, sys->plan.bundles, sys->ia,     \
                                                   sys->ja, a, b, v.x, x_zero, v.r, v.w, dr,    \
                                                   tri ? v.t : nullptr, st, sys->part, sys->hist)
  if (wk == WK_NONE) GB_RESID(WK_NONE);
  else if (wk == WK_JACOBI) GB_RESID(WK_JACOBI);
  else GB_RESID(WK_PREC);
#undef GB_RESID
  GB_CUDA_TRY(cudaGetLastError());
  if (tri) {
    GB_TRY(launch_lower<T>(sys, st, 0, 0, 0));
    GB_TRY(launch_upper<T>(sys, st));
  } else if (wk == WK_PREC) {
    if constexpr (sizeof(T) == 8) {
      GB_TRY(apply_prec_composed(sys, v.r, v.w));
      rho_kernel<T><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(sys->n, v.r, v.w, st, sys->part);
      GB_CUDA_TRY(cudaGetLastError());
    } else {
      return GB_NOT_SUPPORTED;
    }
  }
  return GB_OK;
}

// ------------------------------------------------------------ split precision
// FP64 recurrence (x, r, p, q, the scalars) around the FP32 operator and
// preconditioner: the triangular solves run on the FMA-form FP32 records
// with FP32 outputs t (lower) and s / w (upper).
static int launch_lower_split(gb_system sys, PcgState* st) {
  OpSplitLower<float, double> op{sys->v64.r, sys->v32.s, st, false};
  return tri_launch<float, OpSplitLower<float, double>, false>(
      sys->L32, tri_args<float>(sys->L32, sys->v32.t, sys->err, true), op, sys->s);
}

static int launch_upper_split(gb_system sys, PcgState* st) {
  if (sys->prec == GB_PREC_ICHOL) {
    OpSplitUpper<float> op{sys->v32.t, st, false};
    GB_TRY((tri_launch<float, OpSplitUpper<float>, false>(
        sys->U32, tri_args<float>(sys->U32, sys->v32.s, sys->err, true), op, sys->s)));
    rho_kernel<double, float><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(sys->n, sys->v64.r, sys->v32.s,
                                                                        st, sys->part);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  // GS_std: g = r - A t (v32.r holds g; the split recurrence keeps r in FP64),
  // the sweep, then r'w
  const int nb = sys->plan.nbundles;
  gs_rhs_kernel<float, double><<<wave_grid(gs_rhs_kernel<float, double>, kThreads, ceil_div(nb, kThreads / 32)),
                                 kThreads, 0, sys->s>>>(sys->n, nb, sys->plan.bundles, sys->ia, sys->ja,
                                                        sys->a32, sys->v32.t, sys->v64.r, sys->v32.r, st);
  GB_CUDA_TRY(cudaGetLastError());
  OpSplitGsUpper<float> op{sys->v32.r, sys->v32.t, sys->v32.w, st, false};
  GB_TRY((tri_launch<float, OpSplitGsUpper<float>, false>(
      sys->U32, tri_args<float>(sys->U32, sys->v32.s, sys->err, true), op, sys->s)));
  rho_kernel<double, float><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(sys->n, sys->v64.r, sys->v32.w, st,
                                                                      sys->part);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

static int grid_split(int nb) {
  return wave_grid(spmv_pq_split_kernel, kThreads, ceil_div(nb, kThreads / 32));
}

// w = M^-1 r for the current FP64 r (the lower solve's output is pre-filled
// with the sentinel first); the upper solve rolls rho.
static int apply_prec_split(gb_system sys, PcgState* st) {
  GB_TRY(fill_sentinel_dev(sys->n, sys->v32.t, sys->s));
  GB_TRY(launch_lower_split(sys, st));
  return launch_upper_split(sys, st);
}

int launch_prologue_split(gb_system sys, PcgState* st, const double* b) {
  if (!prec_fused_tri(sys->prec, sys->k)) return GB_NOT_SUPPORTED;
  const int nb = sys->plan.nbundles;
  resid_kernel<double, WK_PREC><<<grid_for_bundles<double>(nb), kThreads, 0, sys->s>>>(
      sys->n, nb, sys->plan.bundles, sys->ia, sys->ja, sys->a, b, sys->v64.x, 0, sys->v64.r,
      nullptr, nullptr, nullptr, st, sys->part, sys->hist);
  GB_CUDA_TRY(cudaGetLastError());
  return apply_prec_split(sys, st);
}

int launch_body_split(gb_system sys, PcgState* st, cudaGraphConditionalHandle cond, int has_cond) {
  if (!prec_fused_tri(sys->prec, sys->k)) return GB_NOT_SUPPORTED;
  auto& v = sys->v64;
  const int nb = sys->plan.nbundles;
  const float* w = sys->prec == GB_PREC_ICHOL ? sys->v32.s : sys->v32.w;
  spmv_pq_split_kernel<<<grid_split(nb), kThreads, 0, sys->s>>>(
      sys->n, nb, sys->plan.bundles, sys->ia, sys->ja, sys->a32, w, v.p0, v.q, sys->v32.t, st,
      sys->part, cond, has_cond);
  GB_CUDA_TRY(cudaGetLastError());
  const double n = sys->n, nz = sys->nnz;
  if (g_prof) prof_mark(sys->s, "spmv_pq_split", nz * 8.0 + (n + 1) * 4.0 + n * (4 + 4 * 8 + 4));
  update_kernel<double, WK_PREC><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(
      sys->n, v.x, v.r, nullptr, v.p0, v.q, nullptr, st, sys->part, sys->hist, cond, has_cond);
  GB_CUDA_TRY(cudaGetLastError());
  if (g_prof) prof_mark(sys->s, "update", 6 * n * 8.0);
  GB_TRY(launch_lower_split(sys, st));
  if (g_prof) prof_mark(sys->s, "lower_solve_split", sys->L32.ndeps * 8.0 + n * 8.0 + n * 8.0 + n * 8.0);
  GB_TRY(launch_upper_split(sys, st));
  if (g_prof)
    prof_mark(sys->s, sys->prec == GB_PREC_ICHOL ? "upper_solve_split" : "gs_upper_solve_split",
              sys->U32.ndeps * 8.0 + n * 8.0 + n * 4.0 + n * 8.0 + n * 4.0 +
                  (sys->prec == GB_PREC_ICHOL ? 0.0 : nz * 8.0 + (n + 1) * 4.0 + n * 8.0));
  return GB_OK;
}

int launch_resume_split(gb_system sys, PcgState* st, double delta) {
  resume_kernel<<<1, 1, 0, sys->s>>>(st, sys->st_out, delta);
  GB_CUDA_TRY(cudaGetLastError());
  return apply_prec_split(sys, st);
}

int launch_outer_resid64(gb_system sys, const double* b, const double* x, int first) {
  const int nb = sys->plan.nbundles;
  outer_resid_kernel<double><<<grid_for_bundles<double>(nb), kThreads, 0, sys->s>>>(
      sys->n, nb, sys->plan.bundles, sys->ia, sys->ja, sys->a, b, x, sys->v64.r, nullptr,
      sys->st_out, sys->part, first);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

template <typename T>
int launch_body(gb_system sys, PcgState* st, cudaGraphConditionalHandle cond, int has_cond) {
  auto v = vecs<T>(sys);
  const int wk = prec_wkind(sys->prec, sys->k);
  const bool tri = prec_fused_tri(sys->prec, sys->k);
  const int nb = sys->plan.nbundles;
  const int g = grid_for_bundles<T>(nb);
  const T* a = mat_vals<T>(sys);
  const T* dr = dr_vals<T>(sys);
  const T* wbuf = w_buffer<T>(sys);
#define GB_PQ(WKV)                                                                             \
  spmv_pq_kernel<T, WKV><<<g, kThreads, 0, sys->s>>>(sys->n, nb, sys->plan.bundles, sys->ia,   \
                                                     sys->ja, a, wbuf, v.p0, v.q,               \
                                                     tri ? v.t : nullptr, st, sys->part, cond,  \
                                                     has_cond)
  if (wk == WK_NONE) GB_PQ(WK_NONE);
  else if (wk == WK_JACOBI) GB_PQ(WK_JACOBI);
  else GB_PQ(WK_PREC);
#undef GB_PQ
  GB_CUDA_TRY(cudaGetLastError());
  // algorithmic bytes: every distinct element touched once, indices 4 B
  const double S = sizeof(T), n = sys->n, nz = sys->nnz;
  const double mat = nz * (4.0 + S) + (n + 1) * 4.0;
  if (g_prof) prof_mark(sys->s, "spmv_pq", mat + 5 * n * S + (tri ? n * S : 0.0));
  if (tri) {
    GB_TRY(launch_lower<T>(sys, st, 1, cond, has_cond));
    if (g_prof)
      prof_mark(sys->s, "lower_solve_update", sys->L.ndeps * (4.0 + S) + n * (S + 4.0) + 8 * n * S);
    GB_TRY(launch_upper<T>(sys, st));
    if (g_prof)
      prof_mark(sys->s, sys->prec == GB_PREC_ICHOL ? "upper_solve_rho" : "gs_upper_solve_rho",
                sys->U.ndeps * (4.0 + S) + n * (S + 4.0) + 3 * n * S +
                    (sys->prec == GB_PREC_ICHOL ? 0.0 : mat + 2 * n * S));
    return GB_OK;
  }
  const int ge = grid_ew(sys->n);
#define GB_UPD(WKV)                                                                            \
  update_kernel<T, WKV><<<ge, kThreads, 0, sys->s>>>(sys->n, v.x, v.r, v.w, v.p0, v.q, dr, st, \
                                                     sys->part, sys->hist, cond, has_cond)
  if (wk == WK_NONE) GB_UPD(WK_NONE);
  else if (wk == WK_JACOBI) GB_UPD(WK_JACOBI);
  else GB_UPD(WK_PREC);
#undef GB_UPD
  GB_CUDA_TRY(cudaGetLastError());
  if (g_prof) prof_mark(sys->s, "update", (wk == WK_JACOBI ? 8 : 6) * n * S);
  if (wk == WK_PREC) {
    if constexpr (sizeof(T) == 8) {
      GB_TRY(apply_prec_composed(sys, v.r, v.w));
      if (g_prof) prof_mark(sys->s, "preconditioner", 0.0);
      rho_kernel<T><<<ge, kThreads, 0, sys->s>>>(sys->n, v.r, v.w, st, sys->part);
      GB_CUDA_TRY(cudaGetLastError());
      if (g_prof) prof_mark(sys->s, "rho", 2 * n * S);
    } else {
      return GB_NOT_SUPPORTED;
    }
  }
  return GB_OK;
}

ProfHook* g_prof = nullptr;

void prof_mark(cudaStream_t s, const char* name, double bytes) {
  ProfHook* h = g_prof;
  if (!h || h->count >= ProfHook::kMax) return;
  h->name[h->count] = name;
  h->bytes[h->count] = bytes;
  cudaEventRecord(h->ev[h->count], s);
  h->count++;
}

template int launch_prologue<double>(gb_system, PcgState*, int, const double*);
template int launch_prologue<float>(gb_system, PcgState*, int, const float*);
template int launch_body<double>(gb_system, PcgState*, cudaGraphConditionalHandle, int);
template int launch_body<float>(gb_system, PcgState*, cudaGraphConditionalHandle, int);

int launch_true_resid(gb_system sys, const double* b, const double* x, double* out2) {
  const int nb = sys->plan.nbundles;
  true_resid_kernel<<<grid_for_bundles<double>(nb), kThreads, 0, sys->s>>>(
      sys->n, nb, sys->plan.bundles, sys->ia, sys->ja, sys->a, b, x, out2, sys->st_out, sys->part);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int launch_outer_resid(gb_system sys, const double* b, const double* x, int first) {
  const int nb = sys->plan.nbundles;
  outer_resid_kernel<float><<<grid_for_bundles<double>(nb), kThreads, 0, sys->s>>>(
      sys->n, nb, sys->plan.bundles, sys->ia, sys->ja, sys->a, b, x, sys->v32.r, sys->v32.x,
      sys->st_out, sys->part, first);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

template <typename T>
int launch_resume(gb_system sys, PcgState* st, double delta) {
  resume_kernel<<<1, 1, 0, sys->s>>>(st, sys->st_out, delta);
  GB_CUDA_TRY(cudaGetLastError());
  auto v = vecs<T>(sys);
  if (prec_fused_tri(sys->prec, sys->k)) {
    // w = M^-1 r for the replaced r; the upper solve rolls rho.  The lower
    // solve's output still holds the last solve's values: refill it with the
    // sentinel, or later tiles would read them as finished.
    GB_TRY(fill_sentinel_dev(sys->n, v.t, sys->s));
    GB_TRY(launch_lower<T>(sys, st, 0, 0, 0));
    return launch_upper<T>(sys, st);
  }
  const int wk = prec_wkind(sys->prec, sys->k);
  if (wk == WK_PREC) return GB_NOT_SUPPORTED;
  if (wk == WK_JACOBI)
    refresh_kernel<T, WK_JACOBI><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(
        sys->n, v.r, v.w, dr_vals<T>(sys), st, sys->part);
  else
    refresh_kernel<T, WK_NONE><<<grid_ew(sys->n), kThreads, 0, sys->s>>>(
        sys->n, v.r, v.w, dr_vals<T>(sys), st, sys->part);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}
template int launch_resume<float>(gb_system, PcgState*, double);
template int launch_resume<double>(gb_system, PcgState*, double);

int launch_add_correction(gb_system sys, double* x) {
  add_correction_kernel<<<grid_ew(sys->n), kThreads, 0, sys->s>>>(sys->n, x, sys->v32.x);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int part_len_needed(gb_system sys) {
  int m = std::max(std::max(grid_for_bundles<double>(sys->plan.nbundles),
                            grid_for_bundles<float>(sys->plan.nbundles)),
                   reduction_grid());
  m = std::max(m, grid_split(sys->plan.nbundles));
  if (sys->tri) m = std::max(m, std::max(std::max(sys->L.ntiles, sys->U.ntiles),
                                         std::max(sys->L32.ntiles, sys->U32.ntiles)));
  return 2 * m + 64;
}

}  // namespace gb
