// batch.cu -- many PCG systems in one persistent CUDA-graph launch.
//
// A batch is S independent systems whose vectors are concatenated:
//   * block-diagonal: S Laplacians of uneven size (gb_batch_create), their
//     CSR concatenated with global row pointers and system-local columns;
//   * multi-RHS: S right-hand sides on one gb_system (gb_pcg_solve_multi),
//     the matrix shared and read once per iteration for all columns; up to
//     32 right-hand sides run on interleaved vectors ([n][S], transposed on
//     entry and exit), more as consecutive chunks of 32 and a shorter last
//     one (the concatenated layout remains as GBLAP_MULTI_FORM=blocks).
// Each system runs its own PCG recurrence of cg.c:42-126 -- its own alpha,
// beta, rho, stopping test and flag -- held in one PcgState per system, so
// the single-system building blocks (pcg_alpha, pcg_check) apply unchanged.
// One iteration of all systems is four launches:
//   bspmv_pq      q = A w + beta q, p = w + beta p; p'q per bundle
//   breduce_alpha per system: p'q in bundle order, alpha (breakdown test)
//   bupdate       x += alpha p, r -= alpha q, w = M^-1 r; r'r, r'w per chunk
//   breduce_check per system: the stopping test; counts the systems still
//                 running and ends the graph's while loop when none is
// Reductions are segmented and in fixed order (partials per bundle / chunk,
// summed by one block per system), so results are reproducible.  A system
// that stopped costs one flag read per bundle.  Preconditioners: line_jacobi
// (y = D^-1 x, line_jacobi.c:3-7) and none.
//
// precision 2 (split): FP32 matrix values and FP32 products A w around the
// FP64 recurrence; a system whose recursive residual has dropped by
// inner_tol (never below its target) pauses, its residual is replaced by the
// FP64 b - A x, and it resumes with p, q and rho kept -- the same scheme as
// the single-system split solve, per system.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "gb_common.cuh"
#include "gblap.h"
#include "kernels.h"
#include "pcg.h"
#include "pcg_state.cuh"
#include "system.h"

namespace gb {

constexpr int kBatchThreads = 256;
constexpr int kBatchWarps = kBatchThreads / 32;
constexpr int kChunkRows = 2048;  // rows of one update / reduction chunk

struct BatchArgs {
  int count, N, n1, nb, nc, shared, jacobi;
  int nbun;             // interleaved: bundles of the shared matrix
  const int* ia;
  const int* ja;
  const int* bundles;   // bundle row starts (global rows, or the shared matrix's rows)
  const int* bsys;      // block-diagonal: system of each bundle
  const int* sys_b;     // block-diagonal: [count+1] bundle range of each system
  const int* chunk_r0;  // [nc+1] chunk row starts (global rows)
  const int* csys;      // [nc] system of each chunk
  const int* sys_c;     // [count+1] chunk range of each system
  const int* row_off;   // [count+1] first row of each system
  const double* a;
  const float* a32;
  const double* d_r;    // [N] (block-diagonal) or [n1] (shared)
  const double* b;
  double *x, *r, *w, *p, *q;
  float* w32;           // interleaved split precision: w rounded once, the FP32 products' operand
  PcgState* st;         // [count] recurrence
  PcgState* so;         // [count] outer (split precision): target and final state
  double* part_b;       // [3 * nb * (shared ? count : 1)]
  double* part_c;       // [2 * nc]
  unsigned* tk;         // [0] check ticket, [1] outer ticket, [2] loop guard
  int* nactive;         // [0] running systems, [1] systems to resume
  int maxit;
  // interleaved split precision: residual replacement inside the loop
  int il_inline;
  int* rep;             // [count] 1 while a system's replacement is being applied
  double delta;         // inner tolerance of a resumed recurrence (relative)
  int max_outer;
};

// x operand of the system whose vectors start at `off`, rounded to the
// matrix's type (FP32 products in the split precision)
template <typename TA>
struct XOff {
  const double* __restrict__ x;
  __device__ __forceinline__ TA operator()(int c) const { return (TA)__ldg(x + c); }
};

__device__ __forceinline__ int sys_bundle_begin(const BatchArgs& B, int s) {
  return B.shared ? s * B.nb : B.sys_b[s];
}
__device__ __forceinline__ int sys_bundle_end(const BatchArgs& B, int s) {
  return B.shared ? (s + 1) * B.nb : B.sys_b[s + 1];
}
__device__ __forceinline__ double dr_at(const BatchArgs& B, int s, int i) {
  return B.shared ? B.d_r[i - s * B.n1] : B.d_r[i];
}

// Runs `body(bundle, s, slot, off)` for every (bundle, system) pair of this
// warp's share: a block-diagonal bundle belongs to one system; a shared-
// matrix bundle is visited once per system, by consecutive warps (system
// fastest), so its entries are read from HBM once and from L1 after that.
template <typename F>
__device__ __forceinline__ void for_bundles(const BatchArgs& B, F&& body) {
  const long long warps = (long long)gridDim.x * kBatchWarps;
  const long long w0 = (long long)blockIdx.x * kBatchWarps + (threadIdx.x >> 5);
  if (!B.shared) {
    for (long long bb = w0; bb < B.nb; bb += warps) body((int)bb, B.bsys[bb], (int)bb, 0);
  } else {
    const long long pairs = (long long)B.nb * B.count;
    for (long long t = w0; t < pairs; t += warps) {
      const int bb = (int)(t / B.count), s = (int)(t % B.count);
      body(bb, s, s * B.nb + bb, s * B.n1);
    }
  }
}

// Fixed-order sum of NV interleaved partials part[stride*i + k], i in
// [i0, i1), by the whole block; valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_segment_sum(const double* part, int stride, int i0, int i1,
                                                  double (&v)[NV], double* sm) {
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += part[(size_t)stride * i + k];
  block_sum<NV>(v, sm);
}

// ------------------------------------------------------------ prologue
// r = b - A x, w = M^-1 r; per bundle: r'r, r'w.
__global__ void __launch_bounds__(kBatchThreads) bresid_kernel(BatchArgs B) {
  __shared__ double stage[kBatchWarps][kBundleNnz];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for_bundles(B, [&](int bb, int s, int slot, int off) {
    struct Ep {
      const BatchArgs& B;
      int s, off;
      double a0, a1;
      __device__ double init(int) const { return 0.0; }
      __device__ void store(int row, double v) {
        const int i = off + row;
        const double ri = B.b[i] - v;
        const double wi = B.jacobi ? dr_at(B, s, i) * ri : ri;
        B.r[i] = ri;
        B.w[i] = wi;
        a0 += ri * ri;
        a1 += ri * wi;
      }
    } ep{B, s, off, 0.0, 0.0};
    XOff<double> xf{B.x + (B.shared ? off : B.row_off[s])};
    spmv_bundle<double, false>(bb, B.shared ? B.n1 : B.N, B.bundles, B.ia, B.ja, B.a, 1.0, xf, ep,
                               stage[wid]);
    const double s0 = warp_sum(ep.a0), s1 = warp_sum(ep.a1);
    if (lane == 0) {
      B.part_b[3 * slot] = s0;
      B.part_b[3 * slot + 1] = s1;
    }
  });
}

// Per system (one block each): ||r0||, the stopping threshold, rho.
__global__ void __launch_bounds__(kBatchThreads) breduce_init_kernel(BatchArgs B) {
  __shared__ double sm[2 * kBatchWarps];
  const int s = blockIdx.x;
  double v[2];
  block_segment_sum<2>(B.part_b, 3, sys_bundle_begin(B, s), sys_bundle_end(B, s), v, sm);
  const double v0 = v[0], v1 = v[1];
  if (threadIdx.x == 0) {
    PcgState& S = B.st[s];
    const double res0 = sqrt(v0);
    S.res0 = res0;
    S.rr = v0;
    S.tolrel = S.spare0 * res0;  // spare0 carries this recurrence's tolerance
    S.rho = B.jacobi ? v1 : v0;
    S.rho_prev = 0.0;
  }
}

// ------------------------------------------------------------ iteration
template <typename TA>
__global__ void __launch_bounds__(kBatchThreads)
    bspmv_pq_kernel(BatchArgs B, const TA* __restrict__ a, cudaGraphConditionalHandle cond, int has_cond) {
  __shared__ TA stage[kBatchWarps][kBundleNnz];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // loop guard, independent of the checking kernel
  if (has_cond && blockIdx.x == 0 && threadIdx.x == 0) {
    const unsigned g = atomicAdd(&B.tk[2], 1u) + 1u;
    if (g > (unsigned)B.maxit + 8u) set_cond(cond, true, false);
  }
  for_bundles(B, [&](int bb, int s, int slot, int off) {
    const PcgState& S = B.st[s];
    if (S.done) return;  // uniform in the warp
    const double beta = S.iter == 0 ? 0.0 : S.rho / S.rho_prev;
    const bool first = S.iter == 0;
    struct Ep {
      const BatchArgs& B;
      int off;
      double beta;
      bool first;
      double pq;
      __device__ TA init(int) const { return TA(0); }
      __device__ void store(int row, TA v) {
        const int i = off + row;
        const double wi = B.w[i];
        const double pi = first ? wi : fma_rn(beta, B.p[i], wi);
        const double qi = first ? (double)v : fma_rn(beta, B.q[i], (double)v);
        B.p[i] = pi;
        B.q[i] = qi;
        pq = fma_rn(pi, qi, pq);
      }
    } ep{B, off, beta, first, 0.0};
    XOff<TA> xf{B.w + (B.shared ? off : B.row_off[s])};
    spmv_bundle<TA, false>(bb, B.shared ? B.n1 : B.N, B.bundles, B.ia, B.ja, a, TA(1), xf, ep,
                           stage[wid]);
    const double v = warp_sum(ep.pq);
    if (lane == 0) B.part_b[3 * slot] = v;
  });
}

__global__ void __launch_bounds__(kBatchThreads) breduce_alpha_kernel(BatchArgs B) {
  __shared__ double sm[kBatchWarps];
  const int s = blockIdx.x;
  PcgState& S = B.st[s];
  if (S.done) return;  // uniform in the block
  double v[1];
  block_segment_sum<1>(B.part_b, 3, sys_bundle_begin(B, s), sys_bundle_end(B, s), v, sm);
  if (threadIdx.x == 0) {
    S.pq = v[0];
    double alpha;
    if (!pcg_alpha(&S, &alpha)) {
      S.done = 1;
      S.flag = 2;
      S.status = GB_BREAKDOWN;
    }
    S.spare1 = alpha;
  }
}

__global__ void __launch_bounds__(kBatchThreads) bupdate_kernel(BatchArgs B) {
  __shared__ double sm[2 * kBatchWarps];
  for (int c = blockIdx.x; c < B.nc; c += gridDim.x) {
    const int s = B.csys[c];
    const PcgState& S = B.st[s];
    if (S.done) continue;  // uniform in the block
    const double al = S.spare1;
    const int r0 = B.chunk_r0[c], r1 = B.chunk_r0[c + 1];
    double acc[2] = {0.0, 0.0};
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
      B.x[i] = fma_rn(al, B.p[i], B.x[i]);
      const double ri = fma_rn(-al, B.q[i], B.r[i]);
      const double wi = B.jacobi ? dr_at(B, s, i) * ri : ri;
      B.r[i] = ri;
      B.w[i] = wi;
      acc[0] = fma_rn(ri, ri, acc[0]);
      acc[1] = fma_rn(ri, wi, acc[1]);
    }
    block_sum<2>(acc, sm);
    if (threadIdx.x == 0) {
      B.part_c[2 * c] = acc[0];
      B.part_c[2 * c + 1] = acc[1];
    }
    __syncthreads();  // sm reused by the next chunk
  }
}

// Counts the systems still running (thread 0 of each live system's block);
// the last block to finish decides whether the loop continues.
__device__ __forceinline__ void batch_loop_decide(const BatchArgs& B, cudaGraphConditionalHandle cond,
                                                  int has_cond) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&B.tk[0], 1u) == gridDim.x - 1u;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    const int live = atomicExch(&B.nactive[0], 0);
    B.nactive[2] = live;  // read by the host-driven (eager) loop
    B.tk[0] = 0u;
    const bool guard_ok = *(volatile unsigned*)&B.tk[2] <= (unsigned)B.maxit + 4u;
    set_cond(cond, has_cond, live > 0 && guard_ok);
    __threadfence();
  }
}

__global__ void __launch_bounds__(kBatchThreads)
    breduce_check_kernel(BatchArgs B, cudaGraphConditionalHandle cond, int has_cond) {
  __shared__ double sm[2 * kBatchWarps];
  const int s = blockIdx.x;
  PcgState& S = B.st[s];
  if (!S.done) {  // uniform in the block
    double v[2];
    block_segment_sum<2>(B.part_c, 2, B.sys_c[s], B.sys_c[s + 1], v, sm);
    if (threadIdx.x == 0) {
      pcg_check(&S, v[0], nullptr);  // hist_len is 0 for batch systems
      if (!S.done) {
        S.rho_prev = S.rho;
        S.rho = B.jacobi ? v[1] : v[0];
        atomicAdd(&B.nactive[0], 1);
      }
    }
  }
  batch_loop_decide(B, cond, has_cond);
}

// ------------------------------------------------------------ true residuals
// replace = 1 (split precision): for every system whose recurrence paused
// converged and is not final, r = b - A x in FP64 and w = M^-1 r (the
// replacement); partials ||r||^2, r'w.  replace = 0 (report): ||b - A x||^2
// and ||b||^2 of every system, nothing written.
__device__ __forceinline__ bool batch_needs_check(const BatchArgs& B, int s) {
  return B.st[s].done && B.st[s].flag == 0 && !B.so[s].done;
}

// Inline replacement: the paused systems are replaced together in a pass
// opened by the loop's decision (nactive[3]), see bil_check_kernel.
__device__ __forceinline__ bool il_replaces(const BatchArgs& B, int s) {
  return B.il_inline && *(volatile int*)&B.nactive[3] && batch_needs_check(B, s);
}

__global__ void __launch_bounds__(kBatchThreads) btrue_kernel(BatchArgs B, int replace) {
  __shared__ double stage[kBatchWarps][kBundleNnz];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for_bundles(B, [&](int bb, int s, int slot, int off) {
    if (replace && !batch_needs_check(B, s)) return;
    struct Ep {
      const BatchArgs& B;
      int s, off, replace;
      double a0, a1, a2;
      __device__ double init(int) const { return 0.0; }
      __device__ void store(int row, double v) {
        const int i = off + row;
        const double bi = B.b[i], ri = bi - v;
        a0 += ri * ri;
        a2 += bi * bi;
        if (replace) {
          const double wi = B.jacobi ? dr_at(B, s, i) * ri : ri;
          B.r[i] = ri;
          B.w[i] = wi;
          a1 += ri * wi;
        }
      }
    } ep{B, s, off, replace, 0.0, 0.0, 0.0};
    XOff<double> xf{B.x + (B.shared ? off : B.row_off[s])};
    spmv_bundle<double, false>(bb, B.shared ? B.n1 : B.N, B.bundles, B.ia, B.ja, B.a, 1.0, xf, ep,
                               stage[wid]);
    const double v0 = warp_sum(ep.a0), v1 = warp_sum(ep.a1), v2 = warp_sum(ep.a2);
    if (lane == 0) {
      B.part_b[3 * slot] = v0;
      B.part_b[3 * slot + 1] = v1;
      B.part_b[3 * slot + 2] = v2;
    }
  });
}

// The refinement decision of a system whose FP64 residual was recomputed
// (||r||^2 = v0, r'w = v1): final when it meets the target (or replacements
// ran out), otherwise the recurrence resumes with the threshold
// max(delta*||r||, target) and rho of the replaced residual (returns true).
__device__ __forceinline__ bool outer_decide(const BatchArgs& B, PcgState& S, PcgState& O, double v0, double v1,
                                             double delta, int max_outer) {
  const double rt = sqrt(v0);
  O.rr = v0;
  O.iter += 1;  // replacements
  if (!(rt == rt) || isinf(rt)) {
    O.done = 1;
    O.flag = 2;
    O.status = GB_BREAKDOWN;
  } else if (rt < O.tolrel) {
    O.done = 1;
    O.flag = 0;
    O.status = GB_OK;
  } else if (O.iter >= max_outer || S.iter > S.maxit) {
    O.done = 1;
    O.flag = 1;
    O.status = GB_MAXIT;
  } else {
    S.done = 0;
    S.flag = 1;
    S.status = GB_OK;
    S.tolrel = fmax(delta * rt, O.tolrel);
    S.rho_prev = S.rho;
    S.rho = B.jacobi ? v1 : v0;
    return true;
  }
  return false;
}

// replace = 1: the refinement decision per checked system -- final when the
// FP64 residual meets the target (or replacements ran out), otherwise the
// recurrence resumes with the threshold max(delta*||r||, target) and rho of
// the replaced residual; nactive[1] counts the resumed systems.
// replace = 0: stores ||b - A x|| in so.spare1 and ||b|| in so.rho.
__global__ void __launch_bounds__(kBatchThreads)
    breduce_outer_kernel(BatchArgs B, int replace, double delta, int max_outer) {
  __shared__ double sm[3 * kBatchWarps];
  const int s = blockIdx.x;
  PcgState& S = B.st[s];
  PcgState& O = B.so[s];
  if (replace && !batch_needs_check(B, s)) {
    // a recurrence that stopped on maxit or breakdown is final as it is
    if (threadIdx.x == 0 && S.done && !O.done) {
      O.done = 1;
      O.flag = S.flag;
      O.status = S.status;
    }
    return;
  }
  double v[3];
  block_segment_sum<3>(B.part_b, 3, sys_bundle_begin(B, s), sys_bundle_end(B, s), v, sm);
  const double v0 = v[0], v1 = v[1], v2 = v[2];
  if (threadIdx.x != 0) return;
  const double rt = sqrt(v0);
  if (!replace) {
    O.spare1 = rt;
    O.rho = sqrt(v2);
    return;
  }
  if (outer_decide(B, S, O, v0, v1, delta, max_outer)) atomicAdd(&B.nactive[1], 1);
}

// target of the refinement: tol * ||b - A x0|| (the recurrence's res0)
__global__ void batch_target_kernel(BatchArgs B) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B.count) return;
  B.so[s].res0 = B.st[s].res0;
  B.so[s].tolrel = B.so[s].spare0 * B.st[s].res0;
}

// 1 / diagonal of every row of a block-diagonal batch (the system-local
// column equal to the row's local index); a missing or zero diagonal is
// reported as its global row + 1.
__global__ void batch_diag_kernel(BatchArgs B, double* d_r, int* bad) {
  for (int c = blockIdx.x; c < B.nc; c += gridDim.x) {
    const int s = B.csys[c], off = B.row_off[s];
    for (int i = B.chunk_r0[c] + threadIdx.x; i < B.chunk_r0[c + 1]; i += blockDim.x) {
      double d = 0.0;
      for (int k = B.ia[i]; k < B.ia[i + 1]; ++k)
        if (B.ja[k] == i - off) d = B.a[k];
      if (d == 0.0) atomicCAS(bad, 0, i + 1);
      d_r[i] = d != 0.0 ? 1.0 / d : 0.0;
    }
  }
}

// ------------------------------------------------------------ interleaved multi-RHS
// Multi-RHS with at most 32 right-hand sides keeps its vectors interleaved,
// v[i * count + s].  A warp takes R = 32 / count rows per step, lane
// sub * count + s serving row sub of the step and right-hand side s: the
// warp's vector accesses are one contiguous run, a row's matrix entries are
// broadcast loads, and a column's values of all right-hand sides are one
// contiguous load.  Every warp sums its rows in order, folds the R rows of a
// right-hand side in lane order and writes part[k + 3 * (s * W + warp)]
// (W = the warps of the grid, the same for every interleaved launch), so the
// per-system reductions above read system s's partials as the contiguous
// range [s W, (s + 1) W) -- a fixed order, hence reproducible results.
enum { IL_RESID = 0, IL_PQ = 1, IL_REPLACE = 2, IL_REPORT = 3 };
constexpr int kIlBatch = 8;  // entries of a row whose loads are in flight together

struct IlLane {
  int C, R, sub, s, W, w0;
  bool ok;  // lanes R * C .. 31 idle
  __device__ IlLane(const BatchArgs& B) {
    const int lane = threadIdx.x & 31;
    C = B.count;
    R = 32 / C;
    sub = lane / C;
    s = lane - sub * C;
    ok = sub < R;
    W = gridDim.x * kBatchWarps;
    w0 = blockIdx.x * kBatchWarps + (threadIdx.x >> 5);
  }
  // sum of v over the R lanes of this lane's right-hand side, valid in sub 0
  __device__ double fold(double v) const {
    const int lane = threadIdx.x & 31;
    double t = v;
    for (int k = 1; k < R; ++k) t += __shfl_sync(0xffffffffu, v, (lane + k * C) & 31);
    return t;
  }
};

// The row kernels walk the shared matrix's SpMV bundles (<= 32 rows), one
// warp per bundle.  Lane t stages row t's entries in shared memory padded to
// kIlSlots slots -- column offsets pre-multiplied by the right-hand-side
// count, padding pointing at the row itself with a zero value -- so each row
// then reads its indices and values with a few 16-byte shared loads and
// issues its kIlSlots gathers without a branch.  A bundle with a row of more
// than kIlSlots entries (or a single long row) is read from global memory.
//
// Split precision (il_inline): a system whose recurrence paused at its
// inner threshold gets its FP64 residual in the next iteration's A w pass:
// its lanes compute r = b - A x with the FP64 values (staged beside the FP32
// ones in such iterations) and x, while the other lanes compute their FP32
// products, so no system waits for the others to pause.
constexpr int kIlSlots = 8;

// FP64 sum of the first N staged products of a row: exactly N gathers and
// N FMAs, since every FP64 instruction -- predicated off or not -- takes a
// slot of GB300's narrow FP64 pipe.
template <int N>
__device__ __forceinline__ double il_chain64(const int* sc_row, const double* sv_row, const double* __restrict__ x,
                                             int s) {
  double xv[N > 0 ? N : 1], acc = 0.0;
#pragma unroll
  for (int u = 0; u < N; ++u) xv[u] = __ldg(x + (unsigned)(sc_row[u] + s));
#pragma unroll
  for (int u = 0; u < N; ++u) acc = fma_rn(sv_row[u], xv[u], acc);
  return acc;
}
__device__ __forceinline__ double il_row64(int cnt, const int* sc_row, const double* sv_row,
                                           const double* __restrict__ x, int s) {
  switch (cnt) {  // uniform in the warp when one row spans it (32 right-hand sides)
    case 8: return il_chain64<8>(sc_row, sv_row, x, s);
    case 7: return il_chain64<7>(sc_row, sv_row, x, s);
    case 6: return il_chain64<6>(sc_row, sv_row, x, s);
    case 5: return il_chain64<5>(sc_row, sv_row, x, s);
    case 4: return il_chain64<4>(sc_row, sv_row, x, s);
    case 3: return il_chain64<3>(sc_row, sv_row, x, s);
    case 2: return il_chain64<2>(sc_row, sv_row, x, s);
    case 1: return il_chain64<1>(sc_row, sv_row, x, s);
    default: return 0.0;
  }
}

template <typename TA, int MODE>
__global__ void __launch_bounds__(kBatchThreads)
    bil_row_kernel(BatchArgs B, const TA* __restrict__ a, cudaGraphConditionalHandle cond, int has_cond) {
  __shared__ __align__(16) int s_col[kBatchWarps][kBundleRows * kIlSlots];
  __shared__ __align__(16) TA s_val[kBatchWarps][kBundleRows * kIlSlots];
  __shared__ int s_cnt[kBatchWarps][kBundleRows];  // entries of each staged row
  constexpr bool kInline = MODE == IL_PQ && sizeof(TA) == 4;
  __shared__ __align__(16) double s_val64[kInline ? kBatchWarps : 1][kInline ? kBundleRows * kIlSlots : 1];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* sc = s_col[wid];
  TA* sv = s_val[wid];
  double* sv64 = s_val64[kInline ? wid : 0];
  const IlLane L(B);
  if (MODE == IL_PQ && has_cond && blockIdx.x == 0 && threadIdx.x == 0) {
    const unsigned g = atomicAdd(&B.tk[2], 1u) + 1u;  // loop guard
    if (g > (unsigned)B.maxit + 8u) set_cond(cond, true, false);
  }
  bool live = false, rep = false, first = false;
  double beta = 0.0;
  if (L.ok) {
    const PcgState& S = B.st[L.s];
    if (MODE == IL_RESID || MODE == IL_REPORT) live = true;
    if (MODE == IL_PQ) {
      live = !S.done;
      first = S.iter == 0;
      beta = first ? 0.0 : S.rho / S.rho_prev;
      if (kInline) rep = il_replaces(B, L.s);
    }
    if (MODE == IL_REPLACE) live = batch_needs_check(B, L.s);
  }
  // the operand A multiplies: w (FP64 or its FP32 copy) or x
  const TA* __restrict__ xs;
  if constexpr (sizeof(TA) == 4) xs = B.w32;
  else xs = MODE == IL_PQ ? B.w : B.x;
  const int C = L.C;
  const bool anyrep = kInline && __any_sync(0xffffffffu, rep);  // uniform in the warp
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  if (__any_sync(0xffffffffu, live || rep)) {
    for (int bb = L.w0; bb < B.nbun; bb += L.W) {
      // a system plan of uniform 32-row bundles has no table (plan-free layout)
      const int r0 = B.bundles ? __ldg(B.bundles + bb) : bb * kBundleRows;
      const int r1 = B.bundles ? __ldg(B.bundles + bb + 1) : min(r0 + kBundleRows, B.n1);
      bool wide = false;
      if (lane < r1 - r0) {
        const int row = r0 + lane, k0 = __ldg(B.ia + row), k1 = __ldg(B.ia + row + 1);
        wide = k1 - k0 > kIlSlots;
        s_cnt[wid][lane] = k1 - k0;
#pragma unroll
        for (int u = 0; u < kIlSlots; ++u) {
          const bool ok = k0 + u < k1;
          sc[lane * kIlSlots + u] = (ok ? __ldg(B.ja + k0 + u) : row) * C;
          sv[lane * kIlSlots + u] = ok ? __ldg(a + k0 + u) : TA(0);
          if (kInline && anyrep) sv64[lane * kIlSlots + u] = ok ? __ldg(B.a + k0 + u) : 0.0;
        }
      }
      const bool fast = !__any_sync(0xffffffffu, wide);  // uniform in the warp
      __syncwarp();
      for (int i = r0 + L.sub; i - L.sub < r1; i += L.R) {
        const bool v = (live || rep) && i < r1;
        const size_t k = (size_t)(v ? i : 0) * C + L.s;
        // own-row operands, loaded before the gathers
        double o0, o1 = 0.0, o2 = 0.0;
        if (MODE == IL_PQ && !rep) {
          o0 = v ? B.w[k] : 0.0;
          o1 = v && !first ? B.p[k] : 0.0;
          o2 = v && !first ? B.q[k] : 0.0;
        } else {
          o0 = v ? B.b[k] : 0.0;
          o1 = v && B.jacobi && MODE != IL_REPORT ? B.d_r[i] : 0.0;
        }
        TA acc = TA(0);
        double acc64 = 0.0;  // inline replacement: FP64 A x
        if (fast) {
          if (v) {
            const int t = (i - r0) * kIlSlots, cnt = s_cnt[wid][i - r0];
            if constexpr (sizeof(TA) == 8) {
              acc = il_row64(cnt, sc + t, sv + t, xs, L.s);
            } else if (!kInline || !rep) {
              // FP32: all slots, padding included, without a branch
              int cc[kIlSlots];
              TA av[kIlSlots], xv[kIlSlots];
#pragma unroll
              for (int u = 0; u < kIlSlots; u += 4) {
                const int4 c4 = *reinterpret_cast<const int4*>(sc + t + u);
                cc[u] = c4.x;
                cc[u + 1] = c4.y;
                cc[u + 2] = c4.z;
                cc[u + 3] = c4.w;
              }
#pragma unroll
              for (int u = 0; u < kIlSlots; ++u) av[u] = sv[t + u];
#pragma unroll
              for (int u = 0; u < kIlSlots; ++u) xv[u] = __ldg(xs + (unsigned)(cc[u] + L.s));
#pragma unroll
              for (int u = 0; u < kIlSlots; ++u) acc = fma_rn(av[u], xv[u], acc);
            } else {
              acc64 = il_row64(cnt, sc + t, sv64 + t, B.x, L.s);
            }
          }
        } else {
          const int e0 = v ? __ldg(B.ia + i) : 0, e1 = v ? __ldg(B.ia + i + 1) : 0;
          for (int e = e0; e < e1; e += kIlBatch) {
            int cc[kIlBatch];
#pragma unroll
            for (int u = 0; u < kIlBatch; ++u) cc[u] = e + u < e1 ? __ldg(B.ja + e + u) : -1;
            if (!kInline || !rep) {
              TA xv[kIlBatch];
#pragma unroll
              for (int u = 0; u < kIlBatch; ++u) xv[u] = cc[u] >= 0 ? __ldg(xs + (size_t)cc[u] * C + L.s) : TA(0);
#pragma unroll
              for (int u = 0; u < kIlBatch; ++u)
                if (cc[u] >= 0) acc = fma_rn(__ldg(a + e + u), xv[u], acc);
            } else {
              double xd[kIlBatch];
#pragma unroll
              for (int u = 0; u < kIlBatch; ++u) xd[u] = cc[u] >= 0 ? __ldg(B.x + (size_t)cc[u] * C + L.s) : 0.0;
#pragma unroll
              for (int u = 0; u < kIlBatch; ++u)
                if (cc[u] >= 0) acc64 = fma_rn(__ldg(B.a + e + u), xd[u], acc64);
            }
          }
        }
        if (!v) continue;
        if (MODE == IL_PQ && !rep) {
          const double wi = o0;
          const double pi = first ? wi : fma_rn(beta, o1, wi);
          const double qi = first ? (double)acc : fma_rn(beta, o2, (double)acc);
          B.p[k] = pi;
          B.q[k] = qi;
          a0 = fma_rn(pi, qi, a0);
        } else {
          const double bi = o0, ri = bi - (rep ? acc64 : (double)acc);
          a0 += ri * ri;
          a2 += bi * bi;
          if (MODE != IL_REPORT) {
            const double wi = B.jacobi ? o1 * ri : ri;
            B.r[k] = ri;
            B.w[k] = wi;
            if (B.w32) B.w32[k] = (float)wi;
            a1 += ri * wi;
          }
        }
      }
      __syncwarp();  // the staging buffers are refilled by the next bundle
    }
  }
  a0 = L.fold(a0);
  if (MODE != IL_PQ || anyrep) {
    a1 = L.fold(a1);
    a2 = L.fold(a2);
  }
  if (L.ok && L.sub == 0 && (live || rep)) {
    const size_t slot = 3 * ((size_t)L.s * L.W + L.w0);
    B.part_b[slot] = a0;
    if (MODE != IL_PQ || rep) {
      B.part_b[slot + 1] = a1;
      B.part_b[slot + 2] = a2;
    }
  }
}

// x += alpha p, r -= alpha q, w = M^-1 r; partials r'r, r'w per (system,
// warp) at part_c[2 * (s * Wu + warp)], Wu = this grid's warps (its own,
// larger than the row kernels').  Each lane takes kIlUpd row steps per pass,
// all their loads issued before any store.
constexpr int kIlUpd = 2;

__global__ void __launch_bounds__(kBatchThreads) bil_update_kernel(BatchArgs B) {
  const IlLane L(B);
  const bool live = L.ok && !B.st[L.s].done && !(B.il_inline && B.rep[L.s]);
  const double al = live ? B.st[L.s].spare1 : 0.0;
  const int C = L.C;
  const double* __restrict__ xv = B.x;
  const double* __restrict__ pv = B.p;
  const double* __restrict__ qv = B.q;
  const double* __restrict__ rv = B.r;
  double a0 = 0.0, a1 = 0.0;
  if (__any_sync(0xffffffffu, live)) {
    const int ng = (B.n1 + L.R - 1) / L.R;
    for (int g = L.w0; g < ng; g += kIlUpd * L.W) {
      double x[kIlUpd], p[kIlUpd], q[kIlUpd], r[kIlUpd], d[kIlUpd];
      bool v[kIlUpd];
      size_t k[kIlUpd];
#pragma unroll
      for (int u = 0; u < kIlUpd; ++u) {
        const int i = (g + u * L.W) * L.R + L.sub;
        v[u] = live && g + u * L.W < ng && i < B.n1;
        k[u] = (size_t)(v[u] ? i : 0) * C + L.s;
        x[u] = v[u] ? xv[k[u]] : 0.0;
        p[u] = v[u] ? pv[k[u]] : 0.0;
        q[u] = v[u] ? qv[k[u]] : 0.0;
        r[u] = v[u] ? rv[k[u]] : 0.0;
        d[u] = v[u] && B.jacobi ? B.d_r[i] : 1.0;
      }
#pragma unroll
      for (int u = 0; u < kIlUpd; ++u) {
        if (!v[u]) continue;
        const double ri = fma_rn(-al, q[u], r[u]);
        const double wi = B.jacobi ? d[u] * ri : ri;
        B.x[k[u]] = fma_rn(al, p[u], x[u]);
        B.r[k[u]] = ri;
        B.w[k[u]] = wi;
        if (B.w32) B.w32[k[u]] = (float)wi;
        a0 = fma_rn(ri, ri, a0);
        a1 = fma_rn(ri, wi, a1);
      }
    }
  }
  a0 = L.fold(a0);
  a1 = L.fold(a1);
  if (L.ok && L.sub == 0 && live) {
    B.part_c[2 * ((size_t)L.s * L.W + L.w0)] = a0;
    B.part_c[2 * ((size_t)L.s * L.W + L.w0) + 1] = a1;
  }
}

// Inline replacement, per system (one block each): alpha of a running
// recurrence, or the refinement decision of a system whose FP64 residual the
// row kernel just recomputed -- marked in rep[s], so that this iteration's
// update skips it and the check counts it without a stopping test.
__global__ void __launch_bounds__(kBatchThreads) bil_alpha_kernel(BatchArgs B) {
  __shared__ double sm[3 * kBatchWarps];
  const int s = blockIdx.x;
  PcgState& S = B.st[s];
  PcgState& O = B.so[s];
  const bool repl = il_replaces(B, s);
  if (!repl && S.done) return;  // uniform in the block
  double v[3];
  block_segment_sum<3>(B.part_b, 3, s * B.nb, (s + 1) * B.nb, v, sm);
  if (threadIdx.x != 0) return;
  if (repl) {
    outer_decide(B, S, O, v[0], v[1], B.delta, B.max_outer);
    B.rep[s] = 1;
    return;
  }
  S.pq = v[0];
  double alpha;
  if (!pcg_alpha(&S, &alpha)) {
    S.done = 1;
    S.flag = 2;
    S.status = GB_BREAKDOWN;
    O.done = 1;
    O.flag = 2;
    O.status = GB_BREAKDOWN;
  }
  S.spare1 = alpha;
}

// Stopping test of the updated systems; a system that paused at its inner
// threshold stays counted (nactive[1] counts those waiting), one that
// stopped on maxit or breakdown is final.  The last block opens a
// replacement pass for all waiting systems (nactive[3]) once all running
// systems have paused, a quarter of the live ones wait, or the first has
// waited kIlWait iterations: each pass costs the whole grid FP64 products,
// so paused systems share one.
constexpr int kIlWait = 4;

__global__ void __launch_bounds__(kBatchThreads)
    bil_check_kernel(BatchArgs B, cudaGraphConditionalHandle cond, int has_cond) {
  __shared__ double sm[2 * kBatchWarps];
  __shared__ int was_rep;
  const int s = blockIdx.x;
  PcgState& S = B.st[s];
  PcgState& O = B.so[s];
  if (threadIdx.x == 0) was_rep = B.rep[s];
  __syncthreads();
  if (was_rep) {
    if (threadIdx.x == 0) {
      B.rep[s] = 0;
      if (!S.done) atomicAdd(&B.nactive[0], 1);  // resumed
    }
  } else if (!S.done) {  // uniform in the block
    double v[2];
    block_segment_sum<2>(B.part_c, 2, B.sys_c[s], B.sys_c[s + 1], v, sm);
    if (threadIdx.x == 0) {
      pcg_check(&S, v[0], nullptr);
      if (!S.done) {
        S.rho_prev = S.rho;
        S.rho = B.jacobi ? v[1] : v[0];
        atomicAdd(&B.nactive[0], 1);
      } else if (S.flag == 0 && !O.done) {
        atomicAdd(&B.nactive[0], 1);
        atomicAdd(&B.nactive[1], 1);
      } else if (!O.done) {
        O.done = 1;
        O.flag = S.flag;
        O.status = S.status;
      }
    }
  } else if (threadIdx.x == 0 && S.flag == 0 && !O.done) {  // still waiting for its pass
    atomicAdd(&B.nactive[0], 1);
    atomicAdd(&B.nactive[1], 1);
  }
  // the last block: the next pass, then the loop's decision
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&B.tk[1], 1u) == gridDim.x - 1u;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    B.tk[1] = 0u;
    const int waiting = atomicExch(&B.nactive[1], 0);
    const int live = *(volatile int*)&B.nactive[0];
    const unsigned waited = waiting > 0 ? B.tk[3] + 1u : 0u;
    const bool go = waiting > 0 && (waiting == live || 4 * waiting >= live || waited >= (unsigned)kIlWait);
    B.nactive[3] = go ? 1 : 0;
    B.tk[3] = go ? 0u : waited;
    __threadfence();
  }
  batch_loop_decide(B, cond, has_cond);
}

// [count][n] -> [n][count] (to_il) or back, 64 rows per tile through shared
// memory, so both the strided and the interleaved side are coalesced.
constexpr int kTrRows = 64;
__global__ void __launch_bounds__(256) bil_transpose_kernel(int n, int C, const double* __restrict__ src,
                                                            double* __restrict__ dst, int to_il) {
  __shared__ double t[32][kTrRows + 1];  // [s][row - i0]
  for (int i0 = blockIdx.x * kTrRows; i0 < n; i0 += gridDim.x * kTrRows) {
    const int rows = min(kTrRows, n - i0);
    if (to_il) {
      for (int e = threadIdx.x; e < C * kTrRows; e += blockDim.x) {
        const int sr = e / kTrRows, r = e - sr * kTrRows;
        if (r < rows) t[sr][r] = src[(size_t)sr * n + i0 + r];
      }
      __syncthreads();
      for (int e = threadIdx.x; e < rows * C; e += blockDim.x) {
        const int r = e / C, sr = e - r * C;
        dst[(size_t)i0 * C + e] = t[sr][r];
      }
    } else {
      for (int e = threadIdx.x; e < rows * C; e += blockDim.x) {
        const int r = e / C, sr = e - r * C;
        t[sr][r] = src[(size_t)i0 * C + e];
      }
      __syncthreads();
      for (int e = threadIdx.x; e < C * kTrRows; e += blockDim.x) {
        const int sr = e / kTrRows, r = e - sr * kTrRows;
        if (r < rows) dst[(size_t)sr * n + i0 + r] = t[sr][r];
      }
    }
    __syncthreads();  // the tile is refilled by the next step
  }
}

}  // namespace gb

// ================================================================ host side
using namespace gb;

struct gb_batch_s {
  int count = 0;
  int shared = 0;  // multi-RHS over one matrix
  int inter = 0;   // multi-RHS with interleaved vectors (count <= 32)
  int N = 0;       // rows of all systems (the vectors' length)
  int n1 = 0;      // rows of the shared matrix
  int jacobi = 1;
  cudaStream_t s = nullptr;
  bool own_stream = false;
  const int* ia = nullptr;
  const int* ja = nullptr;
  const double* a = nullptr;
  const float* a32 = nullptr;
  const double* d_r = nullptr;
  const int* bundles = nullptr;
  int nb = 0, nc = 0;
  int il_grid = 0;  // interleaved: blocks of every row kernel (nb = its warps)
  int il_ugrid = 0; // interleaved: blocks of the update kernel (nc / count = its warps)
  int nbun = 0;     // interleaved: bundles of the shared matrix
  std::vector<void*> owned;  // device buffers freed with the batch
  int *row_off = nullptr, *bsys = nullptr, *sys_b = nullptr, *chunk_r0 = nullptr, *csys = nullptr,
      *sys_c = nullptr;
  double *b = nullptr, *x = nullptr, *r = nullptr, *w = nullptr, *p = nullptr, *q = nullptr;
  float* w32 = nullptr;  // interleaved only
  int* rep = nullptr;    // interleaved only: [count] replacement marks
  int il_inline = 0;     // this solve replaces residuals inside the loop
  double delta = 0.0;    // its inner tolerance
  int max_outer = 0;
  PcgState *st = nullptr, *so = nullptr, *st_h = nullptr;
  double *part_b = nullptr, *part_c = nullptr;
  unsigned* tk = nullptr;
  int* nactive = nullptr;
  LoopGraph loop[2];  // [FP64, split]
  int loop_maxit[2] = {-1, -1};
  int loop_inline[2] = {-1, -1};  // with delta and max_outer: captured in the graph
  double loop_delta[2] = {0.0, 0.0};
  int loop_mo[2] = {-1, -1};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // block-diagonal batches: the host row pointers and system offsets the
  // bundle and chunk tables are (re)built from, the autotuner's choices, and
  // the partial buffers' capacities
  std::vector<int> h_ia, h_roff;
  int rpb = kBundleRows;       // rows per SpMV bundle
  int chunk_rows = kChunkRows; // rows per update / reduction chunk
  size_t part_b_cap = 0, part_c_cap = 0;
};

namespace {

template <typename T>
int balloc(gb_batch bt, T** p, size_t n) {
  void* v = nullptr;
  if (cudaMalloc(&v, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
    cudaGetLastError();
    return GB_NO_MEMORY;
  }
  bt->owned.push_back(v);
  *p = static_cast<T*>(v);
  return GB_OK;
}

template <typename T>
int bupload(gb_batch bt, T** p, const std::vector<T>& h) {
  GB_TRY(balloc(bt, p, h.size()));
  GB_CUDA_TRY(cudaMemcpy(*p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  return GB_OK;
}

void batch_free(gb_batch bt) {
  for (auto& lg : bt->loop) {
    if (lg.exec) cudaGraphExecDestroy(lg.exec);
    if (lg.graph) cudaGraphDestroy(lg.graph);
  }
  for (void* v : bt->owned) cudaFree(v);
  if (bt->st_h) cudaFreeHost(bt->st_h);
  if (bt->ev0) cudaEventDestroy(bt->ev0);
  if (bt->ev1) cudaEventDestroy(bt->ev1);
  if (bt->own_stream && bt->s) cudaStreamDestroy(bt->s);
  delete bt;
}

// Frees a device buffer the batch owns.
void bfree(gb_batch bt, const void* p) {
  if (!p) return;
  auto it = std::find(bt->owned.begin(), bt->owned.end(), const_cast<void*>(p));
  if (it != bt->owned.end()) bt->owned.erase(it);
  cudaFree(const_cast<void*>(p));
}

// Chunks of <= chunk_rows rows, never across systems; row_off on the host.
int batch_chunks(gb_batch bt, const std::vector<int>& row_off) {
  std::vector<int> r0, cs, sc(bt->count + 1, 0);
  for (const void* q : {(const void*)bt->chunk_r0, (const void*)bt->csys, (const void*)bt->sys_c,
                        (const void*)bt->row_off})
    bfree(bt, q);
  bt->chunk_r0 = bt->csys = bt->sys_c = bt->row_off = nullptr;
  for (int s = 0; s < bt->count; ++s) {
    sc[s] = (int)cs.size();
    for (int i = row_off[s]; i < row_off[s + 1]; i += bt->chunk_rows) {
      r0.push_back(i);
      cs.push_back(s);
    }
  }
  sc[bt->count] = (int)cs.size();
  r0.push_back(bt->N);
  bt->nc = (int)cs.size();
  GB_TRY(bupload(bt, &bt->chunk_r0, r0));
  GB_TRY(bupload(bt, &bt->csys, cs));
  GB_TRY(bupload(bt, &bt->sys_c, sc));
  GB_TRY(bupload(bt, &bt->row_off, row_off));
  return GB_OK;
}

// Partial-sum buffers for the current bundle and chunk counts (grown when a
// new plan needs more).
int batch_parts(gb_batch bt) {
  const size_t nb = 3 * (size_t)bt->nb * (bt->shared ? bt->count : 1), nc = 2 * (size_t)bt->nc;
  if (nb > bt->part_b_cap) {
    bfree(bt, bt->part_b);
    GB_TRY(balloc(bt, &bt->part_b, nb));
    bt->part_b_cap = nb;
  }
  if (nc > bt->part_c_cap) {
    bfree(bt, bt->part_c);
    GB_TRY(balloc(bt, &bt->part_c, nc));
    bt->part_c_cap = nc;
  }
  return GB_OK;
}

// Block-diagonal bundles: <= rpb rows and <= kBundleNnz entries of one
// system; a longer row alone.
int batch_bundles(gb_batch bt) {
  const std::vector<int>& hia = bt->h_ia;
  std::vector<int> bun{0}, bsys, sysb(bt->count + 1, 0);
  for (int s = 0; s < bt->count; ++s) {
    sysb[s] = (int)bsys.size();
    int r = bt->h_roff[s];
    const int end = bt->h_roff[s + 1];
    while (r < end) {
      const int start = r;
      long long nz = 0;
      if (hia[r + 1] - hia[r] > kBundleNnz) {
        ++r;
      } else {
        while (r < end && r - start < bt->rpb && nz + (hia[r + 1] - hia[r]) <= kBundleNnz) {
          nz += hia[r + 1] - hia[r];
          ++r;
        }
      }
      bun.push_back(r);
      bsys.push_back(s);
    }
  }
  sysb[bt->count] = (int)bsys.size();
  for (const void* q : {(const void*)bt->bundles, (const void*)bt->bsys, (const void*)bt->sys_b}) bfree(bt, q);
  bt->bundles = nullptr;
  bt->bsys = bt->sys_b = nullptr;
  bt->nb = (int)bsys.size();
  int* dbun = nullptr;
  GB_TRY(bupload(bt, &dbun, bun));
  bt->bundles = dbun;
  GB_TRY(bupload(bt, &bt->bsys, bsys));
  GB_TRY(bupload(bt, &bt->sys_b, sysb));
  return GB_OK;
}

// Vectors, states and partials.
int batch_buffers(gb_batch bt) {
  const size_t N = bt->N;
  for (double** v : {&bt->b, &bt->x, &bt->r, &bt->w, &bt->p, &bt->q}) GB_TRY(balloc(bt, v, N));
  if (bt->inter) GB_TRY(balloc(bt, &bt->w32, N));
  if (bt->inter) GB_TRY(balloc(bt, &bt->rep, bt->count));
  GB_TRY(balloc(bt, &bt->st, bt->count));
  GB_TRY(balloc(bt, &bt->so, bt->count));
  GB_CUDA_TRY(cudaMallocHost(&bt->st_h, sizeof(PcgState) * 2 * bt->count));
  GB_TRY(batch_parts(bt));
  GB_TRY(balloc(bt, &bt->tk, 4));
  GB_TRY(balloc(bt, &bt->nactive, 4));
  GB_CUDA_TRY(cudaMemset(bt->tk, 0, sizeof(unsigned) * 4));
  GB_CUDA_TRY(cudaMemset(bt->nactive, 0, sizeof(int) * 4));
  GB_CUDA_TRY(cudaEventCreate(&bt->ev0));
  GB_CUDA_TRY(cudaEventCreate(&bt->ev1));
  return GB_OK;
}

BatchArgs batch_args(gb_batch bt, int maxit) {
  BatchArgs B;
  memset(&B, 0, sizeof B);
  B.count = bt->count;
  B.N = bt->N;
  B.n1 = bt->n1;
  B.nb = bt->nb;
  B.nbun = bt->nbun;
  B.nc = bt->nc;
  B.shared = bt->shared;
  B.jacobi = bt->jacobi;
  B.ia = bt->ia;
  B.ja = bt->ja;
  B.bundles = bt->bundles;
  B.bsys = bt->bsys;
  B.sys_b = bt->sys_b;
  B.chunk_r0 = bt->chunk_r0;
  B.csys = bt->csys;
  B.sys_c = bt->sys_c;
  B.row_off = bt->row_off;
  B.a = bt->a;
  B.a32 = bt->a32;
  B.d_r = bt->d_r;
  B.b = bt->b;
  B.x = bt->x;
  B.r = bt->r;
  B.w = bt->w;
  B.p = bt->p;
  B.q = bt->q;
  B.st = bt->st;
  B.so = bt->so;
  B.part_b = bt->part_b;
  B.part_c = bt->part_c;
  B.tk = bt->tk;
  B.nactive = bt->nactive;
  B.maxit = maxit;
  B.il_inline = bt->il_inline;
  B.rep = bt->rep;
  B.delta = bt->delta;
  B.max_outer = bt->max_outer;
  return B;
}

int grid_bundles(const void* k, int nb, int count, int shared) {
  const long long warps = (long long)nb * (shared ? count : 1);
  const long long cap = (long long)device_sm_count() * occupancy_blocks(k, kBatchThreads);
  (void)count;
  return (int)std::max(1LL, std::min(cap, (warps + kBatchWarps - 1) / kBatchWarps));
}
int grid_sys(int count) { return count; }  // one block per system
int grid_chunks(int nc) {
  return std::max(1, std::min(nc, device_sm_count() * occupancy_blocks((const void*)bupdate_kernel, kBatchThreads)));
}

template <typename TA, int MODE>
void il_rows(gb_batch bt, const BatchArgs& B, const TA* a, cudaGraphConditionalHandle cond, int has_cond) {
  bil_row_kernel<TA, MODE><<<bt->il_grid, kBatchThreads, 0, bt->s>>>(B, a, cond, has_cond);
}

// One iteration of every live system.
int batch_body(gb_batch bt, int split, int maxit, cudaGraphConditionalHandle cond, int has_cond) {
  BatchArgs B = batch_args(bt, maxit);
  if (split) B.w32 = bt->w32;
  if (bt->inter) {
    if (split) il_rows<float, IL_PQ>(bt, B, bt->a32, cond, has_cond);
    else il_rows<double, IL_PQ>(bt, B, bt->a, cond, has_cond);
    if (B.il_inline) bil_alpha_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B);
    else breduce_alpha_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B);
    bil_update_kernel<<<bt->il_ugrid, kBatchThreads, 0, bt->s>>>(B);
    if (B.il_inline) bil_check_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B, cond, has_cond);
    else breduce_check_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B, cond, has_cond);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  if (split)
    bspmv_pq_kernel<float><<<grid_bundles((const void*)bspmv_pq_kernel<float>, bt->nb, bt->count, bt->shared),
                             kBatchThreads, 0, bt->s>>>(B, bt->a32, cond, has_cond);
  else
    bspmv_pq_kernel<double><<<grid_bundles((const void*)bspmv_pq_kernel<double>, bt->nb, bt->count, bt->shared),
                              kBatchThreads, 0, bt->s>>>(B, bt->a, cond, has_cond);
  GB_CUDA_TRY(cudaGetLastError());
  breduce_alpha_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B);
  bupdate_kernel<<<grid_chunks(bt->nc), kBatchThreads, 0, bt->s>>>(B);
  breduce_check_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B, cond, has_cond);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// The iteration loop as one graph: a while node around batch_body.
int batch_loop(gb_batch bt, int split, int maxit, int use_graph) {
  GB_CUDA_TRY(cudaMemsetAsync(bt->tk, 0, sizeof(unsigned) * 4, bt->s));
  GB_CUDA_TRY(cudaMemsetAsync(bt->nactive, 0, sizeof(int) * 4, bt->s));
  if (!use_graph) {
    for (int it = 0; it <= maxit + 1; it += 16) {
      for (int j = 0; j < 16; ++j) GB_TRY(batch_body(bt, split, maxit, 0, 0));
      int live = 0;
      GB_CUDA_TRY(cudaMemcpyAsync(&live, bt->nactive + 2, sizeof(int), cudaMemcpyDeviceToHost, bt->s));
      GB_CUDA_TRY(cudaStreamSynchronize(bt->s));
      if (live == 0) break;
    }
    return GB_OK;
  }
  LoopGraph& lg = bt->loop[split];
  if (!lg.exec || bt->loop_maxit[split] != maxit || bt->loop_inline[split] != bt->il_inline ||
      bt->loop_delta[split] != bt->delta || bt->loop_mo[split] != bt->max_outer) {
    if (lg.exec) cudaGraphExecDestroy(lg.exec);
    if (lg.graph) cudaGraphDestroy(lg.graph);
    lg = LoopGraph();
    cudaGraph_t g;
    GB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    GB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
    memset(cp_buf, 0, sizeof cp_buf);
    cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cp_buf);
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    GB_CUDA_TRY(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
    GB_CUDA_TRY(cudaStreamBeginCaptureToGraph(bt->s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal));
    const int rc = batch_body(bt, split, maxit, h, 1);
    cudaGraph_t captured = nullptr;
    const cudaError_t e = cudaStreamEndCapture(bt->s, &captured);
    if (rc != GB_OK || e != cudaSuccess) {
      cudaGraphDestroy(g);
      cudaGetLastError();
      return rc != GB_OK ? rc : GB_CUDA_ERROR;
    }
    GB_CUDA_TRY(cudaGraphInstantiate(&lg.exec, g, 0));
    lg.graph = g;
    bt->loop_maxit[split] = maxit;
    bt->loop_inline[split] = bt->il_inline;
    bt->loop_delta[split] = bt->delta;
    bt->loop_mo[split] = bt->max_outer;
  }
  GB_CUDA_TRY(cudaGraphLaunch(lg.exec, bt->s));
  return GB_OK;
}

int batch_solve(gb_batch bt, const double* b, double* x, const gb_pcg_opts* opts, int* iters_host,
                int* flags_host, gb_pcg_result* res) {
  gb_pcg_opts o;
  if (opts) o = *opts;
  else gb_pcg_opts_default(&o);
  if (o.precision != 0 && o.precision != 2) return GB_NOT_SUPPORTED;
  if (o.maxit < 0 || !(o.tol >= 0.0)) return GB_BAD_INPUT;
  const int split = o.precision == 2;
  const double itol = o.inner_tol > 0.0 ? o.inner_tol : 1e-2;
  const size_t bytes = sizeof(double) * (size_t)bt->N;
  PcgState* hs = bt->st_h;
  for (int s = 0; s < bt->count; ++s) {
    PcgState z;
    memset(&z, 0, sizeof z);
    z.flag = 1;
    z.maxit = o.maxit;
    z.spare0 = split ? std::max(itol, o.tol) : o.tol;
    hs[s] = z;
    z.spare0 = o.tol;
    hs[bt->count + s] = z;
  }
  GB_CUDA_TRY(cudaMemcpyAsync(bt->st, hs, sizeof(PcgState) * bt->count, cudaMemcpyHostToDevice, bt->s));
  GB_CUDA_TRY(cudaMemcpyAsync(bt->so, hs + bt->count, sizeof(PcgState) * bt->count, cudaMemcpyHostToDevice, bt->s));
  GB_CUDA_TRY(cudaEventRecord(bt->ev0, bt->s));
  const int gt = std::max(1, std::min(ceil_div(bt->n1, kTrRows), 8 * device_sm_count()));
  if (bt->inter) {
    bil_transpose_kernel<<<gt, 256, 0, bt->s>>>(bt->n1, bt->count, b, bt->b, 1);
    bil_transpose_kernel<<<gt, 256, 0, bt->s>>>(bt->n1, bt->count, x, bt->x, 1);
  } else {
    GB_CUDA_TRY(cudaMemcpyAsync(bt->b, b, bytes, cudaMemcpyDeviceToDevice, bt->s));
    GB_CUDA_TRY(cudaMemcpyAsync(bt->x, x, bytes, cudaMemcpyDeviceToDevice, bt->s));
  }
  // interleaved split precision replaces residuals inside the loop
  bt->il_inline = bt->inter && split;
  bt->delta = itol;
  bt->max_outer = o.max_outer;
  if (bt->il_inline) GB_CUDA_TRY(cudaMemsetAsync(bt->rep, 0, sizeof(int) * bt->count, bt->s));
  BatchArgs B = batch_args(bt, o.maxit);
  if (split) B.w32 = bt->w32;
  const int gb64 = grid_bundles((const void*)bresid_kernel, bt->nb, bt->count, bt->shared);
  if (bt->inter) il_rows<double, IL_RESID>(bt, B, bt->a, 0, 0);
  else bresid_kernel<<<gb64, kBatchThreads, 0, bt->s>>>(B);
  breduce_init_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B);
  batch_target_kernel<<<ceil_div(bt->count, 128), 128, 0, bt->s>>>(B);
  GB_CUDA_TRY(cudaGetLastError());
  // the loop guard allows a replacement pass and its wait per replacement
  GB_TRY(batch_loop(bt, split, bt->il_inline ? o.maxit + o.max_outer * (kIlWait + 1) + 1 : o.maxit, o.use_graph));
  if (split && !bt->il_inline) {
    for (int round = 0; round < o.max_outer + 1; ++round) {
      GB_CUDA_TRY(cudaMemsetAsync(bt->nactive + 1, 0, sizeof(int), bt->s));
      if (bt->inter) il_rows<double, IL_REPLACE>(bt, B, bt->a, 0, 0);
      else btrue_kernel<<<gb64, kBatchThreads, 0, bt->s>>>(B, 1);
      breduce_outer_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B, 1, itol, o.max_outer);
      GB_CUDA_TRY(cudaGetLastError());
      int resumed = 0;
      GB_CUDA_TRY(cudaMemcpyAsync(&resumed, bt->nactive + 1, sizeof(int), cudaMemcpyDeviceToHost, bt->s));
      GB_CUDA_TRY(cudaStreamSynchronize(bt->s));
      if (resumed == 0) break;
      GB_TRY(batch_loop(bt, split, o.maxit, o.use_graph));
    }
  }
  if (bt->inter) il_rows<double, IL_REPORT>(bt, B, bt->a, 0, 0);
  else btrue_kernel<<<gb64, kBatchThreads, 0, bt->s>>>(B, 0);
  breduce_outer_kernel<<<grid_sys(bt->count), kBatchThreads, 0, bt->s>>>(B, 0, itol, o.max_outer);
  GB_CUDA_TRY(cudaGetLastError());
  if (bt->inter) bil_transpose_kernel<<<gt, 256, 0, bt->s>>>(bt->n1, bt->count, bt->x, x, 0);
  else GB_CUDA_TRY(cudaMemcpyAsync(x, bt->x, bytes, cudaMemcpyDeviceToDevice, bt->s));
  GB_CUDA_TRY(cudaEventRecord(bt->ev1, bt->s));
  GB_CUDA_TRY(cudaMemcpyAsync(hs, bt->st, sizeof(PcgState) * bt->count, cudaMemcpyDeviceToHost, bt->s));
  GB_CUDA_TRY(cudaMemcpyAsync(hs + bt->count, bt->so, sizeof(PcgState) * bt->count, cudaMemcpyDeviceToHost, bt->s));
  GB_CUDA_TRY(cudaStreamSynchronize(bt->s));
  gb_pcg_result r;
  memset(&r, 0, sizeof r);
  r.status = GB_OK;
  for (int s = 0; s < bt->count; ++s) {
    const PcgState& S = hs[s];
    const PcgState& O = hs[bt->count + s];
    const int flag = split ? (O.done ? O.flag : 1) : S.flag;
    const int status = split ? (O.done ? O.status : GB_MAXIT) : S.status;
    if (iters_host) iters_host[s] = S.iter;
    if (flags_host) flags_host[s] = flag;
    r.iters = std::max(r.iters, S.iter);
    r.outer = std::max(r.outer, split ? O.iter : 0);
    r.flag = std::max(r.flag, flag);
    if (r.status == GB_OK && status != GB_OK) r.status = status;
    r.res0 = std::max(r.res0, S.res0);
    r.res = std::max(r.res, split ? std::sqrt(O.rr) : std::sqrt(S.rr));
    r.true_res = std::max(r.true_res, O.spare1);
    r.rel_true_res = std::max(r.rel_true_res, O.rho > 0.0 ? O.spare1 / O.rho : O.spare1);
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, bt->ev0, bt->ev1);
  r.device_ms = ms;
  if (res) *res = r;
  return GB_OK;
}

}  // namespace

extern "C" int gb_batch_create(int count, const long long* row_off_host, const long long* nnz_off_host,
                               const int* ia, const int* ja, const double* a, const char* prec_name,
                               gb_batch* out) {
  if (!out || count <= 0 || !row_off_host || !nnz_off_host || !ia || !ja || !a || !prec_name)
    return GB_BAD_INPUT;
  *out = nullptr;
  const int prec = gb_prec_from_name(prec_name);
  if (prec != GB_PREC_LINE_JACOBI && prec != GB_PREC_NONE) return GB_NOT_SUPPORTED;
  if (row_off_host[0] != 0 || nnz_off_host[0] != 0) return GB_BAD_INPUT;
  for (int s = 0; s < count; ++s)
    if (row_off_host[s + 1] <= row_off_host[s] || nnz_off_host[s + 1] < nnz_off_host[s]) return GB_BAD_INPUT;
  if (row_off_host[count] >= (1LL << 31) - 1 || nnz_off_host[count] >= (1LL << 31) - 1) return GB_NOT_SUPPORTED;
  const int N = (int)row_off_host[count];
  std::vector<int> hia(N + 1);
  GB_CUDA_TRY(cudaMemcpy(hia.data(), ia, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost));
  for (int s = 0; s <= count; ++s)
    if (hia[row_off_host[s]] != nnz_off_host[s]) return GB_BAD_INPUT;
  for (int i = 0; i < N; ++i)
    if (hia[i + 1] < hia[i]) return GB_BAD_INPUT;
  gb_batch bt = new gb_batch_s();
  bt->count = count;
  bt->N = N;
  bt->jacobi = prec == GB_PREC_LINE_JACOBI;
  bt->ia = ia;
  bt->ja = ja;
  bt->a = a;
  int rc = GB_OK;
  auto fail = [&](int e) {
    batch_free(bt);
    return e;
  };
  if (cudaStreamCreateWithFlags(&bt->s, cudaStreamNonBlocking) != cudaSuccess) return fail(GB_CUDA_ERROR);
  bt->own_stream = true;
  bt->h_roff.resize(count + 1);
  for (int s = 0; s <= count; ++s) bt->h_roff[s] = (int)row_off_host[s];
  bt->h_ia = std::move(hia);
  if ((rc = batch_bundles(bt)) != GB_OK || (rc = batch_chunks(bt, bt->h_roff)) != GB_OK ||
      (rc = batch_buffers(bt)) != GB_OK)
    return fail(rc);
  // 1/diag and the FP32 values
  const int nnz = (int)nnz_off_host[count];
  double* dr = nullptr;
  float* a32 = nullptr;
  int* bad = nullptr;
  if ((rc = balloc(bt, &dr, N)) != GB_OK || (rc = balloc(bt, &a32, nnz)) != GB_OK ||
      (rc = balloc(bt, &bad, 1)) != GB_OK)
    return fail(rc);
  bt->d_r = dr;
  bt->a32 = a32;
  cudaMemsetAsync(bad, 0, sizeof(int), bt->s);
  batch_diag_kernel<<<grid_chunks(bt->nc), kBatchThreads, 0, bt->s>>>(batch_args(bt, 0), dr, bad);
  if (cast_f64_to_f32(nnz, a, a32, bt->s) != GB_OK) return fail(GB_CUDA_ERROR);
  int hbad = 0;
  if (cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, bt->s) != cudaSuccess ||
      cudaStreamSynchronize(bt->s) != cudaSuccess)
    return fail(GB_CUDA_ERROR);
  if (hbad) return fail(GB_BAD_INPUT);  // a row without a (nonzero) diagonal
  *out = bt;
  return GB_OK;
}

extern "C" int gb_batch_destroy(gb_batch bt) {
  if (!bt) return GB_BAD_INPUT;
  cudaStreamSynchronize(bt->s);
  batch_free(bt);
  return GB_OK;
}

extern "C" int gb_batch_solve(gb_batch bt, const double* b, double* x, const gb_pcg_opts* opts,
                              int* iters_host, int* flags_host, gb_pcg_result* result) {
  if (!bt || !b || !x) return GB_BAD_INPUT;
  return batch_solve(bt, b, x, opts, iters_host, flags_host, result);
}

// Multi-RHS on a gb_system: a shared-matrix batch kept with the system.
namespace gb {
void batch_release(gb_batch bt) {
  if (bt) batch_free(bt);
}
}  // namespace gb

namespace {

// More than this many right-hand sides run as consecutive interleaved
// chunks: one lane per right-hand side in a warp.
constexpr int kIlMaxRhs = 32;

// The shared-matrix batch for nrhs columns in *slot: reused while the count
// and the system's SpMV plan are unchanged, rebuilt otherwise (autotuning
// rebuilds the plan).  interleaved = 0 gives the block form: the columns as
// concatenated vectors, one bundle chunk per column.
int multi_batch(gb_system sys, gb_batch* slot, int nrhs, bool interleaved, gb_batch* out) {
  gb_batch bt = *slot;
  const bool stale = bt && (bt->bundles != sys->plan.bundles ||
                            (bt->inter ? bt->nbun : bt->nb) != sys->plan.nbundles ||
                            (bt->inter != 0) != interleaved);
  if (!bt || bt->count != nrhs || stale) {
    if (bt) batch_free(bt);
    *slot = nullptr;
    bt = new gb_batch_s();
    bt->count = nrhs;
    bt->shared = 1;
    bt->n1 = sys->n;
    bt->N = nrhs * sys->n;
    bt->jacobi = sys->prec == GB_PREC_LINE_JACOBI;
    bt->s = sys->s;
    bt->ia = sys->ia;
    bt->ja = sys->ja;
    bt->a = sys->a;
    bt->a32 = sys->a32;
    bt->d_r = sys->d_r;
    int rc = GB_OK;
    if (interleaved) {
      // interleaved vectors; partials per (right-hand side, warp) of a fixed grid
      bt->inter = 1;
      bt->bundles = sys->plan.bundles;
      bt->nbun = sys->plan.nbundles;
      const long long cap = (long long)device_sm_count() *
                            occupancy_blocks((const void*)bil_row_kernel<double, IL_PQ>, kBatchThreads);
      bt->il_grid = (int)std::max(1LL, std::min(cap, ((long long)bt->nbun + kBatchWarps - 1) / kBatchWarps));
      bt->nb = bt->il_grid * kBatchWarps;
      const long long steps = ((long long)sys->n + 32 / nrhs - 1) / (32 / nrhs);
      bt->il_ugrid = (int)std::max(
          1LL, std::min((long long)device_sm_count() * occupancy_blocks((const void*)bil_update_kernel, kBatchThreads),
                        (steps + kBatchWarps * kIlUpd - 1) / (kBatchWarps * kIlUpd)));
      const int wu = bt->il_ugrid * kBatchWarps;
      bt->nc = wu * nrhs;
      std::vector<int> sc(nrhs + 1);
      for (int s = 0; s <= nrhs; ++s) sc[s] = s * wu;
      if (rc == GB_OK) rc = bupload(bt, &bt->sys_c, sc);
    } else {
      bt->bundles = sys->plan.bundles;
      bt->nb = sys->plan.nbundles;
      std::vector<int> roff(nrhs + 1);
      for (int s = 0; s <= nrhs; ++s) roff[s] = s * sys->n;
      rc = batch_chunks(bt, roff);
    }
    if (rc == GB_OK) rc = batch_buffers(bt);
    if (rc != GB_OK) {
      batch_free(bt);
      return rc;
    }
    *slot = bt;
  }
  *out = bt;
  return GB_OK;
}

}  // namespace

extern "C" int gb_pcg_solve_multi(gb_system sys, int nrhs, const double* B, double* X,
                                  const gb_pcg_opts* opts, int* iters_host, gb_pcg_result* result) {
  if (!sys || nrhs <= 0 || !B || !X) return GB_BAD_INPUT;
  if (sys->prec != GB_PREC_LINE_JACOBI && sys->prec != GB_PREC_NONE) return GB_NOT_SUPPORTED;
  if ((long long)nrhs * sys->n >= (1LL << 31) - 1) return GB_NOT_SUPPORTED;
  // GBLAP_MULTI_FORM=blocks: all columns in one launch as concatenated
  // vectors (the form every count used to take beyond 32)
  const char* form = getenv("GBLAP_MULTI_FORM");
  if (form && !strcmp(form, "blocks")) {
    gb_batch bt = nullptr;
    GB_TRY(multi_batch(sys, &sys->multi, nrhs, false, &bt));
    return batch_solve(bt, B, X, opts, iters_host, nullptr, result);
  }
  const int width = sys->multi_width > 0 ? sys->multi_width : kIlMaxRhs;
  if (nrhs <= width) {
    gb_batch bt = nullptr;
    GB_TRY(multi_batch(sys, &sys->multi, nrhs, true, &bt));
    return batch_solve(bt, B, X, opts, iters_host, nullptr, result);
  }
  // chunks of `width` columns (32 unless the autotuner chose fewer) and a
  // last, shorter one, each an interleaved solve that reads the matrix once
  // per iteration for its columns; the result aggregates the chunks as one
  // solve's does its columns
  gb_pcg_result acc;
  memset(&acc, 0, sizeof acc);
  acc.status = GB_OK;
  const size_t n = (size_t)sys->n;
  for (int c0 = 0; c0 < nrhs; c0 += width) {
    const int c = std::min(width, nrhs - c0);
    gb_batch bt = nullptr;
    GB_TRY(multi_batch(sys, c == width ? &sys->multi : &sys->multi_tail, c, true, &bt));
    gb_pcg_result r;
    GB_TRY(batch_solve(bt, B + (size_t)c0 * n, X + (size_t)c0 * n, opts, iters_host ? iters_host + c0 : nullptr,
                       nullptr, &r));
    acc.iters = std::max(acc.iters, r.iters);
    acc.outer = std::max(acc.outer, r.outer);
    acc.flag = std::max(acc.flag, r.flag);
    if (acc.status == GB_OK && r.status != GB_OK) acc.status = r.status;
    acc.res0 = std::max(acc.res0, r.res0);
    acc.res = std::max(acc.res, r.res);
    acc.true_res = std::max(acc.true_res, r.true_res);
    acc.rel_true_res = std::max(acc.rel_true_res, r.rel_true_res);
    acc.device_ms += r.device_ms;
  }
  if (result) *result = acc;
  return GB_OK;
}

// ------------------------------------------------------------ autotuner
// The batch's tile and row-bundle choices, picked by timing them: each
// candidate runs `iters` iterations of the solve loop the batch really uses
// (the captured CUDA-graph while loop, FP64, tol 0 so no system stops), and
// the fastest is kept.  Choices are cached per matrix class, so a second
// batch of the same shape is tuned without timing.
namespace {
struct BatchClass {
  int count, N, nnz, maxrow;
  bool operator<(const BatchClass& o) const {
    return std::tie(count, N, nnz, maxrow) < std::tie(o.count, o.N, o.nnz, o.maxrow);
  }
};
std::mutex g_btune_mu;
auto& g_btune = *new std::map<BatchClass, std::pair<int, int>>;              // -> (rows per bundle, chunk rows)
auto& g_mtune = *new std::map<std::tuple<int, int, int>, int>;                // (n, nnz, nrhs) -> width

void batch_drop_graphs(gb_batch bt) {
  for (int k = 0; k < 2; ++k) {
    if (bt->loop[k].exec) cudaGraphExecDestroy(bt->loop[k].exec);
    if (bt->loop[k].graph) cudaGraphDestroy(bt->loop[k].graph);
    bt->loop[k] = LoopGraph();
    bt->loop_maxit[k] = -1;
  }
}

int batch_replan(gb_batch bt, int rpb, int chunk_rows) {
  if (rpb == bt->rpb && chunk_rows == bt->chunk_rows) return GB_OK;
  GB_CUDA_TRY(cudaStreamSynchronize(bt->s));
  bt->rpb = rpb;
  bt->chunk_rows = chunk_rows;
  GB_TRY(batch_bundles(bt));
  GB_TRY(batch_chunks(bt, bt->h_roff));
  GB_TRY(batch_parts(bt));
  batch_drop_graphs(bt);
  return GB_OK;
}

// Device time of `iters` FP64 iterations of every system (the first run
// captures the loop graph; the second is timed).
int batch_time(gb_batch bt, const double* b, double* x, int iters, double* ms) {
  gb_pcg_opts o;
  gb_pcg_opts_default(&o);
  o.tol = 0.0;
  o.maxit = iters;
  gb_pcg_result r;
  for (int k = 0; k < 2; ++k) {
    GB_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * (size_t)bt->N, bt->s));
    GB_TRY(batch_solve(bt, b, x, &o, nullptr, nullptr, &r));
  }
  *ms = r.device_ms;
  return GB_OK;
}
}  // namespace

extern "C" int gb_batch_autotune(gb_batch bt, const double* b, int iters, int* rows_per_bundle, int* chunk_rows,
                                 double* ms_default, double* ms_best) {
  if (!bt || !b) return GB_BAD_INPUT;
  if (bt->shared) return GB_NOT_SUPPORTED;  // multi-RHS: gb_pcg_autotune_multi
  if (iters <= 0) iters = 16;
  int maxrow = 0;
  for (int i = 0; i < bt->N; ++i) maxrow = std::max(maxrow, bt->h_ia[i + 1] - bt->h_ia[i]);
  const BatchClass key{bt->count, bt->N, bt->h_ia[bt->N], maxrow};
  std::pair<int, int> best{kBundleRows, kChunkRows};
  double t_def = 0.0, t_best = 0.0;
  bool cached = false;
  {
    std::lock_guard<std::mutex> lk(g_btune_mu);
    auto f = g_btune.find(key);
    if (f != g_btune.end()) {
      best = f->second;
      cached = true;
    }
  }
  if (!cached) {
    double* x = nullptr;
    GB_CUDA_TRY(cudaMalloc(&x, sizeof(double) * std::max(bt->N, 1)));
    int rc = GB_OK;
    t_best = 1e300;
    for (int rpb : {kBundleRows, 16, 8}) {
      for (int cr : {kChunkRows, 1024, 4096}) {
        double ms = 0.0;
        rc = batch_replan(bt, rpb, cr);
        if (rc == GB_OK) rc = batch_time(bt, b, x, iters, &ms);
        if (rc != GB_OK) break;
        if (rpb == kBundleRows && cr == kChunkRows) t_def = ms;
        if (ms < t_best) {
          t_best = ms;
          best = {rpb, cr};
        }
      }
      if (rc != GB_OK) break;
    }
    cudaFree(x);
    if (rc != GB_OK) {
      batch_replan(bt, kBundleRows, kChunkRows);
      return rc;
    }
    std::lock_guard<std::mutex> lk(g_btune_mu);
    g_btune[key] = best;
  }
  GB_TRY(batch_replan(bt, best.first, best.second));
  if (rows_per_bundle) *rows_per_bundle = best.first;
  if (chunk_rows) *chunk_rows = best.second;
  if (ms_default) *ms_default = t_def;
  if (ms_best) *ms_best = t_best;
  return GB_OK;
}

extern "C" int gb_pcg_autotune_multi(gb_system sys, int nrhs, const double* B, int iters, int* width,
                                     double* ms_default, double* ms_best) {
  if (!sys || nrhs <= 0 || !B) return GB_BAD_INPUT;
  if (sys->prec != GB_PREC_LINE_JACOBI && sys->prec != GB_PREC_NONE) return GB_NOT_SUPPORTED;
  if (iters <= 0) iters = 16;
  const auto key = std::make_tuple(sys->n, sys->nnz, nrhs);
  int best = kIlMaxRhs;
  double t_def = 0.0, t_best = 0.0;
  bool cached = false;
  {
    std::lock_guard<std::mutex> lk(g_btune_mu);
    auto f = g_mtune.find(key);
    if (f != g_mtune.end()) {
      best = f->second;
      cached = true;
    }
  }
  if (!cached) {
    double* X = nullptr;
    GB_CUDA_TRY(cudaMalloc(&X, sizeof(double) * (size_t)nrhs * sys->n));
    gb_pcg_opts o;
    gb_pcg_opts_default(&o);
    o.tol = 0.0;
    o.maxit = iters;
    int rc = GB_OK;
    t_best = 1e300;
    const int saved = sys->multi_width;
    for (int w : {kIlMaxRhs, 16, 8}) {
      if (w != kIlMaxRhs && w >= nrhs) continue;  // one chunk either way
      sys->multi_width = w;
      gb_pcg_result r;
      for (int k = 0; k < 2 && rc == GB_OK; ++k) {
        rc = cudaMemsetAsync(X, 0, sizeof(double) * (size_t)nrhs * sys->n, sys->s) == cudaSuccess ? GB_OK
                                                                                                 : GB_CUDA_ERROR;
        if (rc == GB_OK) rc = gb_pcg_solve_multi(sys, nrhs, B, X, &o, nullptr, &r);
      }
      if (rc != GB_OK) break;
      if (w == kIlMaxRhs) t_def = r.device_ms;
      if (r.device_ms < t_best) {
        t_best = r.device_ms;
        best = w;
      }
    }
    sys->multi_width = saved;
    cudaFree(X);
    if (rc != GB_OK) return rc;
    std::lock_guard<std::mutex> lk(g_btune_mu);
    g_mtune[key] = best;
  }
  sys->multi_width = best;
  if (width) *width = best;
  if (ms_default) *ms_default = t_def;
  if (ms_best) *ms_best = t_best;
  return GB_OK;
}
