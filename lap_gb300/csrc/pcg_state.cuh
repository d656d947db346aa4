// pcg_state.cuh -- device-resident PCG recurrence state and the fused
// PCG kernels' building blocks.
#pragma once

#include "gb_common.cuh"
#include "spmv_bundle.cuh"
#include "tri_kernel.cuh"

namespace gb {

// One PCG recurrence (cg.c:42-126) kept in device memory so no scalar ever
// travels to the host during a solve.
struct PcgState {
  double rho;       // r'w of the current iteration  (cg.c:73)
  double rho_prev;  //                                (cg.c:125)
  double pq;        // p'q                            (cg.c:90)
  double rr;        // r'r after the update           (cg.c:102)
  double tolrel;    // tol*||r0||                     (cg.c:60)
  double res0;
  double spare0, spare1;
  int iter;         // completed iterations           (cg.c:101)
  int done;
  int flag;         // 0 converged, 1 maxit, 2 breakdown
  int status;       // gb_status
  int maxit;
  int body_count;   // graph-loop safety counter
  int hist_len;
  int spare_guard;  // bodies started (loop guard in the first body kernel)
  unsigned tk[16];  // reduction tickets, one per kernel kind
};

enum { TK_RESID = 0, TK_PQ = 1, TK_UPD = 2, TK_RHO = 3, TK_TRUE = 4 };

// Applies cg.c's stopping rule after an update.  Called by one thread.
__device__ __forceinline__ void pcg_check(PcgState* st, double rr, double* hist) {
  const double res = sqrt(rr);
  const int it = st->iter + 1;
  st->iter = it;
  st->rr = rr;
  if (it < st->hist_len) hist[it] = res;
  if (!(res == res) || isinf(res)) {
    st->done = 1;
    st->flag = 2;
    st->status = GB_BREAKDOWN;
  } else if (res < st->tolrel) {
    st->done = 1;
    st->flag = 0;
    st->status = GB_OK;
  } else if (it > st->maxit) {
    st->done = 1;
    st->flag = 1;
    st->status = GB_MAXIT;
  }
}

// alpha = rho / p'q with the breakdown test (p'q <= 0 or non-finite).
__device__ __forceinline__ bool pcg_alpha(const PcgState* st, double* alpha) {
  const double pq = st->pq;
  const double a = st->rho / pq;
  *alpha = a;
  return pq > 0.0 && isfinite(a);
}

__device__ __forceinline__ void set_cond(cudaGraphConditionalHandle h, bool has, bool more) {
  if (has) cudaGraphSetConditional(h, more ? 1u : 0u);
}

}  // namespace gb
