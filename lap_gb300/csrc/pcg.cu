// pcg.cu -- the device-resident PCG of cg.c:5-140 with fused kernels.
//
// Per iteration LAP's CUDA build launches ~9 library kernels and reads three
// dot products back to the host (cg.c:73,90,102).  Here one iteration is:
//
//   Jacobi / none : [spmv_pq] [update]                  2 kernels
//   ichol, GS_std : [spmv_pq] [lower solve + update] [upper solve + r'w]
//   others        : [spmv_pq] [update] [LAP preconditioner kernels] [r'w]
//
//   spmv_pq   p_new = w + beta*p_old formed on the fly at every column the
//             row touches (p double-buffered), q = A p_new, p'q reduced;
//   update    x += alpha p, r -= alpha q, r'r and (Jacobi) r'D^-1 r reduced,
//             cg.c's stopping rule applied by the last block;
//
// All scalars (rho, p'q, alpha, beta, the residual history) stay in device
// memory (PcgState); the loop runs as a CUDA-graph while node whose
// condition the checking kernel sets, so a whole solve is one graph launch.
// Elementwise FP64 arithmetic keeps LAP's operation order with explicit
// round-to-nearest mul/add (no FMA contraction), so per-element results
// equal the reference's; only the dot-product summation order differs.
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

template <typename T>
struct VecPtrs {
  T *x, *r, *w, *p0, *p1, *q, *t, *s;
};

// Last-block reduction helper: block sums NV values, publishes, and the last
// block (block-uniform `last`) sums all partials.  Ticket reset by the last.
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

// w at column c for the Jacobi-type preconditioners
template <typename T, int WK>
__device__ __forceinline__ T w_at(const T* __restrict__ r, const T* __restrict__ w,
                                  const T* __restrict__ d_r, int c) {
  if (WK == WK_NONE) return __ldg(r + c);
  if (WK == WK_JACOBI) return mul_rn(__ldg(d_r + c), __ldg(r + c));
  return __ldg(w + c);
}

// ------------------------------------------------------------ prologue
// r = b - A x (x_zero: r = b), r'r, and for Jacobi/none rho = r'w.
// Fills the triangular outputs t (and s) with the sentinel.
template <typename T, int WK>
__global__ void __launch_bounds__(kThreads)
    resid_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                 const int* __restrict__ ja, const T* __restrict__ a, const T* b,
                 const T* __restrict__ x, int x_zero, T* r, const T* __restrict__ d_r, T* tfill,
                 T* sfill, PcgState* st, double* part, double* hist) {
  __shared__ T stage[kThreads / 32][kBundleNnz];
  __shared__ double sm[2 * kThreads / 32];
  const int wid = threadIdx.x >> 5;
  double acc[2] = {0.0, 0.0};
  if (x_zero) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const T ri = b[i];
      r[i] = ri;
      acc[0] += (double)ri * (double)ri;
      if (WK == WK_JACOBI) acc[1] += (double)ri * (double)mul_rn(d_r[i], ri);
      if (tfill) tfill[i] = sentinel<T>();
      if (sfill) sfill[i] = sentinel<T>();
    }
  } else {
    struct Ep {
      const T* b;
      T* r;
      const T* d_r;
      T* tf;
      T* sf;
      double a0, a1;
      __device__ T init(int) const { return T(0); }
      __device__ void store(int i, T v) {
        const T ri = sub_rn(b[i], v);
        r[i] = ri;
        a0 += (double)ri * (double)ri;
        if (WK == WK_JACOBI) a1 += (double)ri * (double)mul_rn(d_r[i], ri);
        if (tf) tf[i] = sentinel<T>();
        if (sf) sf[i] = sentinel<T>();
      }
    } ep{b, r, d_r, tfill, sfill, 0.0, 0.0};
    XPlain<T> xf{x};
    for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
      spmv_bundle(bb, n, bundles, ia, ja, a, T(1), xf, ep, stage[wid]);
    acc[0] = ep.a0;
    acc[1] = ep.a1;
  }
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
template <typename T, int WK>
__global__ void __launch_bounds__(kThreads)
    spmv_pq_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                   const int* __restrict__ ja, const T* __restrict__ a, const T* __restrict__ r,
                   const T* __restrict__ w, const T* __restrict__ d_r, T* p0, T* p1, T* q,
                   T* tfill, PcgState* st, double* part, cudaGraphConditionalHandle cond,
                   int has_cond) {
  __shared__ T stage[kThreads / 32][kBundleNnz];
  __shared__ double sm[kThreads / 32];
  // Loop guard, independent of the checking kernel later in the body: a
  // graph while loop can never run more than maxit + 8 bodies.
  if (has_cond && blockIdx.x == 0 && threadIdx.x == 0) {
    const int g = ++st->spare_guard;
    if (g > st->maxit + 8) set_cond(cond, true, false);
  }
  if (st->done) return;  // uniform across the grid
  const int it = st->iter;
  const bool first = it == 0;
  const T beta = first ? T(0) : (T)(st->rho / st->rho_prev);
  const T* __restrict__ pold = (it & 1) ? p1 : p0;
  T* pnew = (it & 1) ? p0 : p1;
  struct XF {
    const T *r, *w, *d_r, *pold;
    T beta;
    bool first;
    __device__ T operator()(int c) const {
      const T wc = w_at<T, WK>(r, w, d_r, c);
      return first ? wc : add_rn(mul_rn(beta, __ldg(pold + c)), wc);
    }
  } xf{r, w, d_r, pold, beta, first};
  struct Ep {
    XF* xf;
    T *pnew, *q, *tf;
    double pq;
    __device__ T init(int) const { return T(0); }
    __device__ void store(int i, T v) {
      const T pi = (*xf)(i);
      pnew[i] = pi;
      q[i] = v;
      pq += (double)pi * (double)v;
      if (tf) tf[i] = sentinel<T>();
    }
  } ep{&xf, pnew, q, tfill, 0.0};
  const int wid = threadIdx.x >> 5;
  for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
    spmv_bundle(bb, n, bundles, ia, ja, a, T(1), xf, ep, stage[wid]);
  double acc[1] = {ep.pq};
  if (reduce_last<1>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_PQ], sm) && threadIdx.x == 0)
    st->pq = acc[0];
}

// ------------------------------------------------------------ update
template <typename T, int WK>
__global__ void __launch_bounds__(kThreads)
    update_kernel(int n, T* x, T* r, const T* __restrict__ p0, const T* __restrict__ p1,
                  const T* __restrict__ q, const T* __restrict__ d_r, PcgState* st, double* part,
                  double* hist, cudaGraphConditionalHandle cond, int has_cond) {
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
  const int it = st->iter;
  const T* __restrict__ p = (it & 1) ? p0 : p1;  // p_new of this iteration
  const T a = (T)alpha, na = (T)(-alpha);
  double acc[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = add_rn(x[i], mul_rn(a, p[i]));
    const T ri = add_rn(r[i], mul_rn(na, q[i]));
    r[i] = ri;
    acc[0] += (double)ri * (double)ri;
    if (WK == WK_JACOBI) acc[1] += (double)ri * (double)mul_rn(d_r[i], ri);
  }
  if (reduce_last<2>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_UPD], sm) && threadIdx.x == 0) {
    pcg_check(st, acc[0], hist);
    if (WK != WK_PREC) {
      st->rho_prev = st->rho;
      st->rho = WK == WK_NONE ? acc[0] : acc[1];
    }
    set_cond(cond, has_cond, !st->done && st->body_count++ < st->maxit + 4);
  }
}

// rho = r'w after a composed preconditioner (PREC kind)
template <typename T>
__global__ void __launch_bounds__(kThreads)
    rho_kernel(int n, const T* __restrict__ r, const T* __restrict__ w, PcgState* st,
               double* part) {
  __shared__ double sm[kThreads / 32];
  if (st->done) return;
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc[0] += (double)r[i] * (double)w[i];
  if (reduce_last<1>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_RHO], sm) && threadIdx.x == 0) {
    st->rho_prev = st->rho;
    st->rho = acc[0];
  }
}

// ------------------------------------------------------------ fused tri ops
// Lower solve with the x/r update fused in front (do_update) -- the update
// of row i is elementwise, and row i's right-hand side is r_i only.
template <typename T>
struct OpPcgLower {
  T *x, *r;
  const T *p0, *p1, *q;
  T* sfill;
  PcgState* st;
  double* part;
  double* hist;
  cudaGraphConditionalHandle cond;
  int has_cond, do_update;
  // per thread
  bool dn, ok;
  T a, na;
  const T* p;
  double rr;
  __device__ void begin() {
    dn = st->done != 0;
    ok = true;
    rr = 0.0;
    if (do_update && !dn) {
      double alpha;
      ok = pcg_alpha(st, &alpha);
      a = (T)alpha;
      na = (T)(-alpha);
      p = (st->iter & 1) ? p0 : p1;
    }
  }
  __device__ bool active() const { return !dn && ok; }
  __device__ T rhs(int i) {
    if (!do_update) return r[i];
    x[i] = add_rn(x[i], mul_rn(a, p[i]));
    const T ri = add_rn(r[i], mul_rn(na, q[i]));
    r[i] = ri;
    rr += (double)ri * (double)ri;
    return ri;
  }
  __device__ void done(int i, T) {
    if (sfill) sfill[i] = sentinel<T>();
  }
  __device__ void block_end(int bid, int nblocks, unsigned* ticket, double* sm) {
    double v[1] = {rr};
    block_sum<1>(v, sm);
    __shared__ bool last;
    if (threadIdx.x == 0) {
      part[bid] = v[0];
      __threadfence();
      last = atomicAdd(&ticket[1], 1u) == (unsigned)nblocks - 1u;
      if (last) {
        ticket[0] = 0u;
        ticket[1] = 0u;
        __threadfence();
      }
    }
    __syncthreads();
    if (!last || !do_update) return;
    double t[1] = {0.0};
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) t[0] += ld_relaxed(part + i);
    block_sum<1>(t, sm);
    if (threadIdx.x == 0) {
      if (dn) {
        set_cond(cond, has_cond, false);
      } else if (!ok) {
        st->done = 1;
        st->flag = 2;
        st->status = GB_BREAKDOWN;
        set_cond(cond, has_cond, false);
      } else {
        pcg_check(st, t[0], hist);
        set_cond(cond, has_cond, !st->done && st->body_count++ < st->maxit + 4);
      }
    }
  }
};

// Upper solve whose output is w (ichol: w = (L L^T)^-1 r), reducing r'w.
template <typename T>
struct OpIcUpper {
  const T* t;
  const T* r;
  PcgState* st;
  double* part;
  bool dn;
  double rho;
  __device__ void begin() {
    dn = st->done != 0;
    rho = 0.0;
  }
  __device__ bool active() const { return !dn; }
  __device__ T rhs(int i) const { return t[i]; }
  __device__ void done(int i, T y) { rho += (double)r[i] * (double)y; }
  __device__ void block_end(int bid, int nblocks, unsigned* ticket, double* sm) {
    double v[1] = {rho};
    block_sum<1>(v, sm);
    __shared__ bool last;
    if (threadIdx.x == 0) {
      part[bid] = v[0];
      __threadfence();
      last = atomicAdd(&ticket[1], 1u) == (unsigned)nblocks - 1u;
      if (last) {
        ticket[0] = 0u;
        ticket[1] = 0u;
        __threadfence();
      }
    }
    __syncthreads();
    if (!last) return;
    double s[1] = {0.0};
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) s[0] += ld_relaxed(part + i);
    block_sum<1>(s, sm);
    if (threadIdx.x == 0 && !dn) {
      st->rho_prev = st->rho;
      st->rho = s[0];
    }
  }
};

// GS_std (k = 1) backward sweep: rhs_i = r_i - (A t)_i in LAP's order
// (GS.c:34-35: copy then csr_matvec(-1, 1)), y = (D+U)^-1 rhs,
// w = t + y (GS.c:40), reducing r'w.
template <typename T>
struct OpGsUpper {
  const T* t;
  const T* r;
  const int* ia;
  const int* ja;
  const T* av;
  T* w;
  PcgState* st;
  double* part;
  bool dn;
  double rho;
  __device__ void begin() {
    dn = st->done != 0;
    rho = 0.0;
  }
  __device__ bool active() const { return !dn; }
  __device__ T rhs(int i) const {
    T acc = r[i];
    for (int j = ia[i]; j < ia[i + 1]; ++j) acc = add_rn(acc, mul_rn(-av[j], t[ja[j]]));
    return acc;
  }
  __device__ void done(int i, T y) {
    const T wi = add_rn(t[i], y);
    w[i] = wi;
    rho += (double)r[i] * (double)wi;
  }
  __device__ void block_end(int bid, int nblocks, unsigned* ticket, double* sm) {
    OpIcUpper<T> tmp{nullptr, nullptr, st, part, dn, rho};
    tmp.block_end(bid, nblocks, ticket, sm);
  }
};

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
      const double ri = sub_rn(b[i], v);
      a0 += ri * ri;
      a1 += b[i] * b[i];
    }
  } ep{b, 0.0, 0.0};
  XPlain<double> xf{x};
  const int wid = threadIdx.x >> 5;
  for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
    spmv_bundle(bb, n, bundles, ia, ja, a, 1.0, xf, ep, stage[wid]);
  double acc[2] = {ep.a0, ep.a1};
  if (reduce_last<2>(acc, part, gridDim.x, blockIdx.x, &st->tk[TK_TRUE], sm) && threadIdx.x == 0) {
    out2[0] = sqrt(acc[0]);
    out2[1] = sqrt(acc[1]);
  }
}

// ------------------------------------------------------------ mixed precision helpers
// Outer FP64 residual r = b - A x, its norm, cast to the FP32 inner rhs, and
// the refinement stopping test against tol * ||b - A x0||.
__global__ void __launch_bounds__(kThreads)
    outer_resid_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                       const int* __restrict__ ja, const double* __restrict__ a,
                       const double* __restrict__ b, const double* __restrict__ x, float* r32,
                       float* x32, PcgState* so, double* part, int first) {
  __shared__ double stage[kThreads / 32][kBundleNnz];
  __shared__ double sm[kThreads / 32];
  struct Ep {
    const double* b;
    float *r32, *x32;
    double a0;
    __device__ double init(int) const { return 0.0; }
    __device__ void store(int i, double v) {
      const double ri = sub_rn(b[i], v);
      r32[i] = (float)ri;
      x32[i] = 0.0f;
      a0 += ri * ri;
    }
  } ep{b, r32, x32, 0.0};
  XPlain<double> xf{x};
  const int wid = threadIdx.x >> 5;
  for (int bb = blockIdx.x * (kThreads / 32) + wid; bb < nb; bb += gridDim.x * (kThreads / 32))
    spmv_bundle(bb, n, bundles, ia, ja, a, 1.0, xf, ep, stage[wid]);
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

// ================================================================ host side
static int grid_for_bundles(int nb) {
  return std::max(1, std::min(ceil_div(nb, kThreads / 32), device_sm_count() * 8));
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

template <typename T>
static TriArgs<T> tri_args(const TriPlan& p, T* y, int* err) {
  TriArgs<T> A;
  A.nwarps = p.nwarps;
  A.slot_row = p.slot_row;
  A.warp_ptr = p.warp_ptr;
  A.warp_len = p.warp_len;
  A.ecol = p.ecol;
  if constexpr (sizeof(T) == 8) {
    A.eval = (const T*)p.eval;
    A.diag = (const T*)p.diag;
  } else {
    A.eval = (const T*)p.eval32;
    A.diag = (const T*)p.diag32;
  }
  A.y = y;
  A.ticket = p.ticket;
  A.err = err;
  return A;
}

// Launches the fused lower solve (prologue: do_update = 0).
template <typename T>
static int launch_lower(gb_system sys, PcgState* st, int do_update, cudaGraphConditionalHandle cond,
                        int has_cond) {
  auto v = vecs<T>(sys);
  OpPcgLower<T> op{};
  op.x = v.x;
  op.r = v.r;
  op.p0 = v.p0;
  op.p1 = v.p1;
  op.q = v.q;
  op.sfill = v.s;
  op.st = st;
  op.part = sys->part;
  op.hist = sys->hist;
  op.cond = cond;
  op.has_cond = has_cond;
  op.do_update = do_update;
  const int blocks = ceil_div(sys->L.nwarps, kTriWarps);
  tri_solve_kernel<T, OpPcgLower<T>><<<blocks, kTriWarps * 32, 0, sys->s>>>(
      tri_args<T>(sys->L, v.t, sys->err), op);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

template <typename T>
static int launch_upper(gb_system sys, PcgState* st) {
  auto v = vecs<T>(sys);
  const int blocks = ceil_div(sys->U.nwarps, kTriWarps);
  if (sys->prec == GB_PREC_ICHOL) {
    OpIcUpper<T> op{v.t, v.r, st, sys->part, false, 0.0};
    tri_solve_kernel<T, OpIcUpper<T>><<<blocks, kTriWarps * 32, 0, sys->s>>>(
        tri_args<T>(sys->U, v.s, sys->err), op);
  } else {
    OpGsUpper<T> op{v.t, v.r, sys->ia, sys->ja, mat_vals<T>(sys), v.w, st, sys->part, false, 0.0};
    tri_solve_kernel<T, OpGsUpper<T>><<<blocks, kTriWarps * 32, 0, sys->s>>>(
        tri_args<T>(sys->U, v.s, sys->err), op);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// w buffer the spmv_pq kernel reads: ichol writes w into the upper solve's
// output s; GS_std and the composed preconditioners into w.
template <typename T>
static const T* w_buffer(gb_system sys) {
  auto v = vecs<T>(sys);
  return sys->prec == GB_PREC_ICHOL ? v.s : v.w;
}

template <typename T>
int launch_prologue(gb_system sys, PcgState* st, int x_zero, const T* b) {
  auto v = vecs<T>(sys);
  const int wk = prec_wkind(sys->prec, sys->k);
  const bool tri = prec_fused_tri(sys->prec, sys->k);
  const int nb = sys->plan.nbundles;
  const int g = grid_for_bundles(nb);
  const T* a = mat_vals<T>(sys);
  const T* dr = dr_vals<T>(sys);
#define GB_RESID(WKV)                                                                           \
  resid_kernel<T, WKV><<<g, kThreads, 0, sys->s>>>(sys->n, nb, sys->plan.bundles, sys->ia,      \
                                                   sys->ja, a, b, v.x, x_zero, v.r, dr,          \
                                                   tri ? v.t : nullptr, nullptr, st, sys->part,  \
                                                   sys->hist)
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

template <typename T>
int launch_body(gb_system sys, PcgState* st, cudaGraphConditionalHandle cond, int has_cond) {
  auto v = vecs<T>(sys);
  const int wk = prec_wkind(sys->prec, sys->k);
  const bool tri = prec_fused_tri(sys->prec, sys->k);
  const int nb = sys->plan.nbundles;
  const int g = grid_for_bundles(nb);
  const T* a = mat_vals<T>(sys);
  const T* dr = dr_vals<T>(sys);
  const T* wbuf = w_buffer<T>(sys);
#define GB_PQ(WKV)                                                                              \
  spmv_pq_kernel<T, WKV><<<g, kThreads, 0, sys->s>>>(sys->n, nb, sys->plan.bundles, sys->ia,    \
                                                     sys->ja, a, v.r, wbuf, dr, v.p0, v.p1, v.q, \
                                                     tri ? v.t : nullptr, st, sys->part, cond,   \
                                                     has_cond)
  if (wk == WK_NONE) GB_PQ(WK_NONE);
  else if (wk == WK_JACOBI) GB_PQ(WK_JACOBI);
  else GB_PQ(WK_PREC);
#undef GB_PQ
  GB_CUDA_TRY(cudaGetLastError());
  // algorithmic bytes: every distinct element touched once, indices 4 B
  const double S = sizeof(T), n = sys->n, nz = sys->nnz;
  const double mat = nz * (4.0 + S) + (n + 1) * 4.0;
  if (g_prof) prof_mark(sys->s, "spmv_pq", mat + (wk == WK_JACOBI ? 3 : 2) * n * S + (tri ? 3 : 2) * n * S);
  if (tri) {
    GB_TRY(launch_lower<T>(sys, st, 1, cond, has_cond));
    if (g_prof)
      prof_mark(sys->s, "lower_solve_update",
                sys->L.ndeps * (4.0 + S) + n * (S + 4.0) + 8 * n * S);
    GB_TRY(launch_upper<T>(sys, st));
    if (g_prof)
      prof_mark(sys->s, sys->prec == GB_PREC_ICHOL ? "upper_solve_rho" : "gs_upper_solve_rho",
                sys->U.ndeps * (4.0 + S) + n * (S + 4.0) + 3 * n * S +
                    (sys->prec == GB_PREC_ICHOL ? 0.0 : mat + n * S));
    return GB_OK;
  }
  const int ge = grid_ew(sys->n);
#define GB_UPD(WKV)                                                                             \
  update_kernel<T, WKV><<<ge, kThreads, 0, sys->s>>>(sys->n, v.x, v.r, v.p0, v.p1, v.q, dr, st, \
                                                     sys->part, sys->hist, cond, has_cond)
  if (wk == WK_NONE) GB_UPD(WK_NONE);
  else if (wk == WK_JACOBI) GB_UPD(WK_JACOBI);
  else GB_UPD(WK_PREC);
#undef GB_UPD
  GB_CUDA_TRY(cudaGetLastError());
  if (g_prof) prof_mark(sys->s, "update", (wk == WK_JACOBI ? 7 : 6) * n * S);
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
  true_resid_kernel<<<grid_for_bundles(nb), kThreads, 0, sys->s>>>(
      sys->n, nb, sys->plan.bundles, sys->ia, sys->ja, sys->a, b, x, out2, sys->st_out, sys->part);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int launch_outer_resid(gb_system sys, const double* b, const double* x, int first) {
  const int nb = sys->plan.nbundles;
  outer_resid_kernel<<<grid_for_bundles(nb), kThreads, 0, sys->s>>>(
      sys->n, nb, sys->plan.bundles, sys->ia, sys->ja, sys->a, b, x, sys->v32.r, sys->v32.x,
      sys->st_out, sys->part, first);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int launch_add_correction(gb_system sys, double* x) {
  add_correction_kernel<<<grid_ew(sys->n), kThreads, 0, sys->s>>>(sys->n, x, sys->v32.x);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int part_len_needed(gb_system sys) {
  int m = std::max(grid_for_bundles(sys->plan.nbundles), reduction_grid());
  if (sys->tri) m = std::max(m, std::max(ceil_div(sys->L.nwarps, kTriWarps), ceil_div(sys->U.nwarps, kTriWarps)));
  return 2 * m + 64;
}

}  // namespace gb
