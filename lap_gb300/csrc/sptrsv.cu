// sptrsv.cu -- dependency lists of the triangular factors (host) and the
// on-device IC(0) factorization (replacing cusparseDcsric02,
// cuda_blas.cu:261-488).  The tiled solve schedule is in tri_plan.cu.
#include <algorithm>
#include <vector>

#include "gb_common.cuh"
#include "kernels.h"
#include "sptrsv.h"
#include "spmv_bundle.cuh"

namespace gb {

// ------------------------------------------------------------ dependency lists
int deps_embedded(int n, const int* ia, const int* ja, bool lower, TriDeps* d) {
  d->n = n;
  d->lower = lower;
  d->row_ptr.assign(n + 1, 0);
  d->diag_src.assign(n, -1);
  d->dep_col.clear();
  d->dep_src.clear();
  d->dep_col.reserve(ia[n]);
  d->dep_src.reserve(ia[n]);
  for (int i = 0; i < n; ++i) {
    for (int k = ia[i]; k < ia[i + 1]; ++k) {
      const int c = ja[k];
      if (c == i) {
        d->diag_src[i] = k;
      } else {
        if ((lower && c > i) || (!lower && c < i) || c < 0 || c >= n) return GB_BAD_INPUT;
        d->dep_col.push_back(c);
        d->dep_src.push_back(k);
      }
    }
    if (d->diag_src[i] < 0) return GB_BAD_INPUT;
    d->row_ptr[i + 1] = (int)d->dep_col.size();
  }
  return GB_OK;
}

int deps_strict(int n, const int* ia, const int* ja, bool lower, TriDeps* d) {
  d->n = n;
  d->lower = lower;
  d->row_ptr.assign(ia, ia + n + 1);
  const int m = ia[n] - ia[0];
  d->dep_col.assign(ja + ia[0], ja + ia[0] + m);
  d->dep_src.resize(m);
  for (int k = 0; k < m; ++k) {
    d->dep_src[k] = ia[0] + k;
    const int c = d->dep_col[k];
    if (c < 0 || c >= n) return GB_BAD_INPUT;
  }
  if (ia[0] != 0)
    for (auto& p : d->row_ptr) p -= ia[0];
  for (int i = 0; i < n; ++i)
    for (int k = d->row_ptr[i]; k < d->row_ptr[i + 1]; ++k)
      if ((lower && d->dep_col[k] >= i) || (!lower && d->dep_col[k] <= i)) return GB_BAD_INPUT;
  d->diag_src.resize(n);
  for (int i = 0; i < n; ++i) d->diag_src[i] = i;
  return GB_OK;
}

int transpose_positions(int n, const int* ia, const int* ja, std::vector<int>* tpos) {
  const int nnz = ia[n];
  tpos->assign(nnz, -1);
  std::vector<int> next(ia, ia + n);
  for (int i = 0; i < n; ++i) {
    for (int k = ia[i]; k < ia[i + 1]; ++k) {
      const int j = ja[k];
      if (j < 0 || j >= n) return GB_BAD_INPUT;
      const int p = next[j]++;
      if (p >= ia[j + 1] || ja[p] != i) return GB_BAD_INPUT;  // pattern not symmetric
      (*tpos)[k] = p;
    }
  }
  return GB_OK;
}

int deps_ichol(int n, const int* ia, const int* ja, const std::vector<int>& tpos, bool lower,
               TriDeps* d) {
  d->n = n;
  d->lower = lower;
  d->row_ptr.assign(n + 1, 0);
  d->diag_src.assign(n, -1);
  d->dep_col.clear();
  d->dep_src.clear();
  for (int i = 0; i < n; ++i) {
    for (int k = ia[i]; k < ia[i + 1]; ++k) {
      const int c = ja[k];
      if (c == i) {
        d->diag_src[i] = k;
      } else if (lower && c < i) {
        d->dep_col.push_back(c);
        d->dep_src.push_back(k);  // L_ic stored at (i, c)
      } else if (!lower && c > i) {
        d->dep_col.push_back(c);
        d->dep_src.push_back(tpos[k]);  // (L^T)_ic = L_ci stored at (c, i)
      }
    }
    if (d->diag_src[i] < 0) return GB_BAD_INPUT;
    d->row_ptr[i + 1] = (int)d->dep_col.size();
  }
  return GB_OK;
}

// ------------------------------------------------------------ IC(0) factor
// Left-looking restatement of simple_blas.c:139-168: row j receives, for
// every i < j with (i, j) in the pattern and in increasing i, the update
// a_jc -= u_ij * u_ic for each c >= j shared by rows i and j -- exactly the
// updates, in exactly the order, that the reference's right-looking sweep
// applies to row j -- then u_jj = sqrt(a_jj) and u_jc = a_jc / u_jj.
//
// One warp per row.  The dependencies i are taken one after another (each
// entry of row j sees its updates in the reference's order, so the factor
// is bit-identical); within one dependency the lanes split row i's upper
// entries and find each column in row j by bisection (columns are sorted
// and unique, so no two lanes update the same entry).  A hub row with
// thousands of dependencies thus costs thousands of short warp steps, not
// millions of serial merge steps.  Rows run in global level order, taken in
// groups of one block's warps by ticket (a group never spans two levels: the
// order pads every level to a multiple of 32); a row waits for its
// dependencies' done flags (acquire) and publishes its own (release).
constexpr int kFactorWarps = 8;
// Rows whose upper part is longer than kSkipMin entries search it through a
// coarse index in shared memory first: every stride-th column (at most
// kSkip of them), so a lookup costs ~10 shared-memory steps and then a
// bisection inside one window of stride entries (one or two cache lines)
// instead of ~17 dependent loads across the whole row.  Power-law hub rows
// (tens of thousands of entries, each updated by tens of thousands of
// dependencies) are what this is for.
constexpr int kSkip = 1024;
constexpr int kSkipMin = 256;
static_assert(32 % kFactorWarps == 0, "a group must lie inside one padded level");
// Wall-clock limit of one wait in the factorization: a power-law graph's hub
// rows carry tens of thousands of dependencies each and chain through one
// another, so a row may legitimately wait seconds for a hub.  A limit set
// with gb_debug_set_spin_budget takes precedence.
constexpr uint64_t kFactorWaitNs = 120ull * 1000000000ull;

// Acquire-poll of a done flag with the factorization's limit (all lanes poll
// the same word); false on timeout or when another wait already failed.
__device__ __forceinline__ bool factor_wait(const int* flag, int* err) {
  if (ld_acquire(flag) != 0) return true;
  const uint64_t dbg = *reinterpret_cast<const volatile unsigned long long*>(err + 2);
  const uint64_t budget = dbg ? dbg : kFactorWaitNs;
  const uint64_t t0 = globaltimer_ns();
  unsigned polls = 0, ns = 32u;
  while (true) {
    __nanosleep(ns);
    if (ns < kMaxSleepNs) ns <<= 1;
    if (ld_acquire(flag) != 0) return true;
    if ((++polls & kPollCheck) == 0u && (ld_volatile(err) != 0 || globaltimer_ns() - t0 > budget)) {
      atomicCAS(err, 0, (int)GB_TIMEOUT);
      return false;
    }
  }
}

__global__ void __launch_bounds__(kFactorWarps * 32)
    ichol_factor_kernel(int norder, const int* __restrict__ order, const int* __restrict__ ia,
                        const int* __restrict__ ja, const int* __restrict__ dpos,
                        const int* __restrict__ tpos, double* f, int* done, unsigned* ticket,
                        int* zero_pivot, int* err) {
  __shared__ int s_group;
  __shared__ int s_skip[kFactorWarps][kSkip];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ngroups = ceil_div(norder, kFactorWarps);
  while (true) {
    if (threadIdx.x == 0) s_group = (int)atomicAdd(&ticket[0], 1u);
    __syncthreads();
    const int group = s_group;
    __syncthreads();
    if (group >= ngroups) break;
    const int slot = group * kFactorWarps + wid;
    const int j = slot < norder ? order[slot] : -1;
    if (j < 0) continue;  // level padding (warp-uniform)
    const int d = dpos[j], je = ia[j + 1];
    bool ok = true;
    // coarse index of row j's upper columns (long rows only)
    const int ulen = je - d;
    int stride = 0, nsk = 0;
    if (ulen > kSkipMin) {
      stride = max(32, (ulen + kSkip - 1) / kSkip);
      nsk = (ulen + stride - 1) / stride;
      __syncwarp();  // the previous row's lookups are done with s_skip
      for (int q = lane; q < nsk; q += 32) s_skip[wid][q] = ja[d + q * stride];
      __syncwarp();
    }
    // dependencies i = ja[k] < j, ascending, 32 at a time: lane t reads the
    // done flag (acquire), u_ij and row i's end of dependency k0 + t in
    // parallel; a dependency not finished yet is then awaited in its turn
    for (int k0 = ia[j]; k0 < d && ok; k0 += 32) {
      const int kl = k0 + lane;
      const int il = kl < d ? ja[kl] : -1;
      const int ml = kl < d ? tpos[kl] : 0;
      const int ready_l = il < 0 ? 1 : ld_acquire(done + il);
      const double ul = (il >= 0 && ready_l) ? __ldcg(f + ml) : 0.0;
      const int iel = il >= 0 ? ia[il + 1] : 0;
      __syncwarp();  // lanes' acquires order every lane's later reads of those rows
      const int nk = min(32, d - k0);
      for (int t = 0; t < nk; ++t) {
        const int i = __shfl_sync(0xffffffffu, il, t);
        const int m = __shfl_sync(0xffffffffu, ml, t);  // (i, j) inside row i's upper part
        const int ie = __shfl_sync(0xffffffffu, iel, t);
        double uij = __shfl_sync(0xffffffffu, ul, t);
        if (!__shfl_sync(0xffffffffu, ready_l, t)) {
          ok = __all_sync(0xffffffffu, factor_wait(done + i, err));
          if (!ok) break;
          // row i was written by another SM: read it through L2 (ld.global.cg)
          uij = __ldcg(f + m);
        }
        for (int l = m + lane; l < ie; l += 32) {
          const int c = ja[l];
          int lo = d, hi = je - 1;  // bisection for column c in row j's upper part
          if (stride) {
            // the last index entry <= c (entry 0 is j itself, and c >= j)
            int a = 0, b = nsk - 1;
            while (a < b) {
              const int mid = (a + b + 1) >> 1;
              if (s_skip[wid][mid] <= c) a = mid;
              else b = mid - 1;
            }
            lo = d + a * stride;
            hi = min(lo + stride - 1, je - 1);
          }
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (ja[mid] < c) lo = mid + 1;
            else hi = mid;
          }
          if (ja[lo] == c) f[lo] = sub_rn(f[lo], mul_rn(uij, __ldcg(f + l)));
        }
        __syncwarp();  // this dependency's updates land before the next one's
      }
    }
    if (!ok) continue;  // timed out: the row stays unpublished, dependents time out too
    const double piv = f[d];
    if (!(piv > 0.0) && lane == 0) atomicCAS(zero_pivot, 0, j + 1);
    const double u = __dsqrt_rn(piv);
    __syncwarp();
    if (lane == 0) f[d] = u;
    for (int kk = d + 1 + lane; kk < je; kk += 32) {
      const double v = __ddiv_rn(f[kk], u);
      f[kk] = v;
      f[tpos[kk]] = v;  // symmetric copy: L_cj = U_jc
    }
    __threadfence();  // every lane's writes of row j before the flag
    __syncwarp();
    if (lane == 0) st_release(done + j, 1);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ticket[2], 1u) == gridDim.x - 1u) {
      ticket[0] = 0u;
      ticket[2] = 0u;
      __threadfence();
    }
  }
}

__global__ void ichol_init_kernel(int nnz, const double* __restrict__ a, double* f, int n,
                                  int* done) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) f[i] = a[i];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) done[i] = 0;
}

int ichol_factor_dev(int n, const int* ia, const int* ja, const double* a, const int* dpos,
                     const int* tpos, const TriPlan* lp, double* f, int* done, unsigned* ticket,
                     int* zero_pivot, int* err, cudaStream_t s) {
  if (n <= 0) return GB_OK;
  int nnz = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&nnz, ia + n, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  const int g = std::max(1, std::min(device_sm_count() * 8, ceil_div(std::max(nnz, n), 256)));
  ichol_init_kernel<<<g, 256, 0, s>>>(nnz, a, f, n, done);
  GB_CUDA_TRY(cudaMemsetAsync(zero_pivot, 0, sizeof(int), s));
  const int per_sm = occupancy_blocks((const void*)ichol_factor_kernel, kFactorWarps * 32);
  const int blocks = std::max(1, std::min(ceil_div(lp->norder, kFactorWarps), device_sm_count() * per_sm));
  ichol_factor_kernel<<<blocks, kFactorWarps * 32, 0, s>>>(lp->norder, lp->order, ia, ja, dpos, tpos, f,
                                                           done, ticket, zero_pivot, err);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
