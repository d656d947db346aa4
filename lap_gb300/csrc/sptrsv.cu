// sptrsv.cu -- host-side level scheduling for the sync-free triangular
// solves (replacing csrsv2 analysis, cuda_blas.cu:99-224) and the on-device
// IC(0) factorization (replacing cusparseDcsric02, cuda_blas.cu:261-488).
#include <algorithm>
#include <vector>

#include "gb_common.cuh"
#include "kernels.h"
#include "sptrsv.h"
#include "tri_kernel.cuh"

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

// ------------------------------------------------------------ schedule
template <typename V>
static int upload(V** dst, const std::vector<V>& src) {
  const size_t bytes = sizeof(V) * std::max<size_t>(src.size(), 1);
  GB_CUDA_TRY(cudaMalloc(dst, bytes));
  if (!src.empty()) GB_CUDA_TRY(cudaMemcpy(*dst, src.data(), sizeof(V) * src.size(), cudaMemcpyHostToDevice));
  return GB_OK;
}

int tri_plan_build(const TriDeps& d, TriPlan* plan) {
  const int n = d.n;
  std::vector<int> lev(n, 0);
  int nlev = 0;
  if (d.lower) {
    for (int i = 0; i < n; ++i) {
      int l = 0;
      for (int k = d.row_ptr[i]; k < d.row_ptr[i + 1]; ++k) l = std::max(l, lev[d.dep_col[k]] + 1);
      lev[i] = l;
      nlev = std::max(nlev, l + 1);
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int l = 0;
      for (int k = d.row_ptr[i]; k < d.row_ptr[i + 1]; ++k) l = std::max(l, lev[d.dep_col[k]] + 1);
      lev[i] = l;
      nlev = std::max(nlev, l + 1);
    }
  }
  // counting sort by level, rows ascending within a level
  std::vector<int> lptr(nlev + 1, 0);
  for (int i = 0; i < n; ++i) lptr[lev[i] + 1]++;
  for (int l = 0; l < nlev; ++l) lptr[l + 1] += lptr[l];
  std::vector<int> byl(n), fill(lptr.begin(), lptr.end() - 1);
  for (int i = 0; i < n; ++i) byl[fill[lev[i]]++] = i;

  std::vector<int> slot_row, warp_ptr, warp_len, ecol, emap, dmap;
  warp_ptr.push_back(0);
  std::vector<int> shortrows;
  for (int l = 0; l < nlev; ++l) {
    shortrows.clear();
    std::vector<int> longrows;
    for (int p = lptr[l]; p < lptr[l + 1]; ++p) {
      const int r = byl[p];
      (d.row_ptr[r + 1] - d.row_ptr[r] > 32 ? longrows : shortrows).push_back(r);
    }
    for (size_t s0 = 0; s0 < shortrows.size(); s0 += 32) {
      const int cnt = (int)std::min<size_t>(32, shortrows.size() - s0);
      int len = 0;
      for (int t = 0; t < cnt; ++t) {
        const int r = shortrows[s0 + t];
        len = std::max(len, d.row_ptr[r + 1] - d.row_ptr[r]);
      }
      const int base = (int)ecol.size();
      ecol.resize(base + (size_t)len * 32, -1);
      emap.resize(base + (size_t)len * 32, -1);
      for (int t = 0; t < 32; ++t) {
        const int r = t < cnt ? shortrows[s0 + t] : -1;
        slot_row.push_back(r);
        dmap.push_back(r >= 0 ? d.diag_src[r] : -1);
        if (r < 0) continue;
        for (int k = d.row_ptr[r], q = 0; k < d.row_ptr[r + 1]; ++k, ++q) {
          ecol[base + q * 32 + t] = d.dep_col[k];
          emap[base + q * 32 + t] = d.dep_src[k];
        }
      }
      warp_len.push_back(len);
      warp_ptr.push_back((int)ecol.size());
    }
    for (int r : longrows) {
      const int base = (int)ecol.size();
      for (int k = d.row_ptr[r]; k < d.row_ptr[r + 1]; ++k) {
        ecol.push_back(d.dep_col[k]);
        emap.push_back(d.dep_src[k]);
      }
      slot_row.push_back(r);
      dmap.push_back(d.diag_src[r]);
      for (int t = 1; t < 32; ++t) {
        slot_row.push_back(-1);
        dmap.push_back(-1);
      }
      warp_len.push_back(-(d.row_ptr[r + 1] - d.row_ptr[r]));
      warp_ptr.push_back((int)ecol.size());
      (void)base;
    }
  }
  plan->n = n;
  plan->lower = d.lower;
  plan->nlevels = nlev;
  plan->nwarps = (int)warp_len.size();
  plan->nent = (int)ecol.size();
  plan->ndeps = (long long)d.dep_col.size();
  GB_TRY(upload(&plan->slot_row, slot_row));
  GB_TRY(upload(&plan->warp_ptr, warp_ptr));
  GB_TRY(upload(&plan->warp_len, warp_len));
  GB_TRY(upload(&plan->ecol, ecol));
  GB_TRY(upload(&plan->emap, emap));
  GB_TRY(upload(&plan->dmap, dmap));
  GB_CUDA_TRY(cudaMalloc(&plan->eval, sizeof(double) * std::max(1, plan->nent)));
  GB_CUDA_TRY(cudaMalloc(&plan->diag, sizeof(double) * std::max(1, plan->nwarps * 32)));
  GB_CUDA_TRY(cudaMalloc(&plan->ticket, sizeof(unsigned) * 4));
  GB_CUDA_TRY(cudaMemset(plan->ticket, 0, sizeof(unsigned) * 4));
  return GB_OK;
}

void tri_plan_free(TriPlan* p) {
  void* ptrs[] = {p->slot_row, p->warp_ptr, p->warp_len, p->ecol, p->emap, p->dmap,
                  p->eval,     p->diag,     p->eval32,   p->diag32, p->ticket};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  *p = TriPlan();
}

int tri_plan_fill(TriPlan* p, const double* ent_src, const double* diag_src, bool want32,
                  cudaStream_t s) {
  if (want32 && !p->eval32) {
    GB_CUDA_TRY(cudaMalloc(&p->eval32, sizeof(float) * std::max(1, p->nent)));
    GB_CUDA_TRY(cudaMalloc(&p->diag32, sizeof(float) * std::max(1, p->nwarps * 32)));
  }
  GB_TRY(gather_values(p->nent, p->emap, ent_src, p->eval, want32 ? p->eval32 : nullptr, s));
  GB_TRY(gather_values(p->nwarps * 32, p->dmap, diag_src, p->diag, want32 ? p->diag32 : nullptr, s));
  return GB_OK;
}

template <typename T>
int tri_solve_plain(const TriPlan* p, const T* x, T* y, int* err, cudaStream_t s) {
  if (p->n <= 0) return GB_OK;
  GB_TRY(fill_sentinel_dev(p->n, y, s));
  TriArgs<T> A;
  A.nwarps = p->nwarps;
  A.slot_row = p->slot_row;
  A.warp_ptr = p->warp_ptr;
  A.warp_len = p->warp_len;
  A.ecol = p->ecol;
  if constexpr (sizeof(T) == 8) {
    A.eval = (const T*)p->eval;
    A.diag = (const T*)p->diag;
  } else {
    A.eval = (const T*)p->eval32;
    A.diag = (const T*)p->diag32;
  }
  A.y = y;
  A.ticket = p->ticket;
  A.err = err;
  OpPlain<T> op{x};
  const int blocks = ceil_div(p->nwarps, kTriWarps);
  tri_solve_kernel<T, OpPlain<T>><<<blocks, kTriWarps * 32, 0, s>>>(A, op);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}
template int tri_solve_plain<double>(const TriPlan*, const double*, double*, int*, cudaStream_t);
template int tri_solve_plain<float>(const TriPlan*, const float*, float*, int*, cudaStream_t);

// ------------------------------------------------------------ IC(0) factor
// Left-looking restatement of simple_blas.c:139-168: row j receives, for
// every i < j with (i, j) in the pattern and in increasing i, the update
// a_jc -= u_ij * u_ic for each c >= j shared by rows i and j -- exactly the
// updates, in exactly the order, that the reference's right-looking sweep
// applies to row j -- then u_jj = sqrt(a_jj) and u_jc = a_jc / u_jj.  Rows
// run in the lower schedule's level order; row j waits for its dependencies'
// done flags (acquire) and publishes its own (release).
__global__ void __launch_bounds__(kTriWarps * 32)
    ichol_factor_kernel(int nslots, const int* __restrict__ slot_row, const int* __restrict__ ia,
                        const int* __restrict__ ja, const int* __restrict__ dpos,
                        const int* __restrict__ tpos, double* f, int* done, unsigned* ticket,
                        int* zero_pivot, int* err) {
  __shared__ int s_bid;
  if (threadIdx.x == 0) s_bid = (int)atomicAdd(&ticket[0], 1u);
  __syncthreads();
  const int slot = s_bid * (kTriWarps * 32) + threadIdx.x;
  const int j = slot < nslots ? slot_row[slot] : -1;
  if (j >= 0) {
    const int d = dpos[j], je = ia[j + 1];
    for (int k = ia[j]; k < d; ++k) {  // dependencies i = ja[k] < j, ascending
      const int i = ja[k];
      if (!wait_flag(done + i, err)) break;
      const int m = tpos[k];  // (i, j) inside row i's upper part
      // row i was written by another SM: read it through L2 (ld.global.cg)
      const double uij = __ldcg(f + m);
      int l = m, kk = d;
      const int ie = ia[i + 1];
      while (l < ie && kk < je) {
        const int cl = ja[l], ck = ja[kk];
        if (cl == ck) {
          f[kk] = sub_rn(f[kk], mul_rn(uij, __ldcg(f + l)));
          ++l;
          ++kk;
        } else if (cl < ck) {
          ++l;
        } else {
          ++kk;
        }
      }
    }
    const double piv = f[d];
    if (!(piv > 0.0)) atomicCAS(zero_pivot, 0, j + 1);
    const double u = __dsqrt_rn(piv);
    f[d] = u;
    for (int kk = d + 1; kk < je; ++kk) {
      const double v = __ddiv_rn(f[kk], u);
      f[kk] = v;
      f[tpos[kk]] = v;  // symmetric copy: L_cj = U_jc
    }
    __threadfence();
    st_release(done + j, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ticket[1], 1u) == gridDim.x - 1u) {
      ticket[0] = 0u;
      ticket[1] = 0u;
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
  const int nslots = lp->nwarps * 32;
  const int blocks = ceil_div(nslots, kTriWarps * 32);
  ichol_factor_kernel<<<blocks, kTriWarps * 32, 0, s>>>(nslots, lp->slot_row, ia, ja, dpos, tpos,
                                                         f, done, ticket, zero_pivot, err);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
