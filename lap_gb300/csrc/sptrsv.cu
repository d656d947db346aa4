// sptrsv.cu -- host-side scheduling for the tiled sync-free triangular
// solves (replacing csrsv2 analysis, cuda_blas.cu:99-224) and the on-device
// IC(0) factorization (replacing cusparseDcsric02, cuda_blas.cu:261-488).
#include <algorithm>
#include <cstdlib>
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

int tri_default_tile_rows(int n) {
  // one tile per SM when the matrix is large; at least 1024 rows, at most
  // 16384 (128 KB of FP64 shared memory)
  const int sms = device_sm_count();
  int t = 1024;
  while (t < 16384 && (long long)t * sms < n) t <<= 1;
  return t;
}

int tri_plan_build(const TriDeps& d, TriPlan* plan, int tile_rows) {
  const int n = d.n;
  const bool lower = d.lower;
  if (tile_rows <= 0) tile_rows = tri_default_tile_rows(n);
  tile_rows = std::max(32, std::min(tile_rows, 16384));
  auto deps_of = [&](int r) { return d.row_ptr[r + 1] - d.row_ptr[r]; };

  // global levels: the IC(0) factorization order and a diagnostic
  std::vector<int> lev(n, 0);
  int nlev = 0;
  for (int q = 0; q < n; ++q) {
    const int i = lower ? q : n - 1 - q;
    int l = 0;
    for (int k = d.row_ptr[i]; k < d.row_ptr[i + 1]; ++k) l = std::max(l, lev[d.dep_col[k]] + 1);
    lev[i] = l;
    nlev = std::max(nlev, l + 1);
  }
  std::vector<int> order;
  {
    std::vector<int> lptr(nlev + 1, 0);
    for (int i = 0; i < n; ++i) lptr[lev[i] + 1]++;
    for (int l = 0; l < nlev; ++l) lptr[l + 1] += lptr[l];
    std::vector<int> byl(n), fill(lptr.begin(), lptr.end() - 1);
    for (int i = 0; i < n; ++i) byl[fill[lev[i]]++] = i;
    for (int l = 0; l < nlev; ++l) {
      for (int p = lptr[l]; p < lptr[l + 1]; ++p) order.push_back(byl[p]);
      while (order.size() % 32) order.push_back(-1);
    }
  }

  // tiles, local levels, slices
  const int ntiles = (n + tile_rows - 1) / tile_rows;
  std::vector<int> tr0, tr1, tile_lvl{0}, lvl_slice{0}, slice_rows, slice_ent, slice_len, ecol, emap, dmap;
  std::vector<int> llev(tile_rows), bucket_ptr, bucket;
  for (int q = 0; q < ntiles; ++q) {
    const int tix = lower ? q : ntiles - 1 - q;
    const int t0 = tix * tile_rows, t1 = std::min(n, t0 + tile_rows);
    tr0.push_back(t0);
    tr1.push_back(t1);
    int nl = 0;
    for (int s = 0; s < t1 - t0; ++s) {
      const int i = lower ? t0 + s : t1 - 1 - s;
      int l = 0;
      for (int k = d.row_ptr[i]; k < d.row_ptr[i + 1]; ++k) {
        const int c = d.dep_col[k];
        if (c >= t0 && c < t1) l = std::max(l, llev[c - t0] + 1);
      }
      llev[i - t0] = l;
      nl = std::max(nl, l + 1);
    }
    bucket_ptr.assign(nl + 1, 0);
    for (int i = t0; i < t1; ++i) bucket_ptr[llev[i - t0] + 1]++;
    for (int l = 0; l < nl; ++l) bucket_ptr[l + 1] += bucket_ptr[l];
    bucket.resize(t1 - t0);
    std::vector<int> fill(bucket_ptr.begin(), bucket_ptr.end() - 1);
    for (int i = t0; i < t1; ++i) bucket[fill[llev[i - t0]]++] = i;
    for (int l = 0; l < nl; ++l) {
      std::vector<int> shortrows, longrows;
      for (int p = bucket_ptr[l]; p < bucket_ptr[l + 1]; ++p)
        (deps_of(bucket[p]) > 32 ? longrows : shortrows).push_back(bucket[p]);
      for (size_t s0 = 0; s0 < shortrows.size(); s0 += 32) {
        const int cnt = (int)std::min<size_t>(32, shortrows.size() - s0);
        int len = 0;
        for (int t = 0; t < cnt; ++t) len = std::max(len, deps_of(shortrows[s0 + t]));
        const int base = (int)ecol.size();
        ecol.resize(base + (size_t)len * 32, -1);
        emap.resize(base + (size_t)len * 32, -1);
        for (int t = 0; t < 32; ++t) {
          const int r = t < cnt ? shortrows[s0 + t] : -1;
          slice_rows.push_back(r);
          dmap.push_back(r >= 0 ? d.diag_src[r] : -1);
          if (r < 0) continue;
          for (int k = d.row_ptr[r], e = 0; k < d.row_ptr[r + 1]; ++k, ++e) {
            ecol[base + e * 32 + t] = d.dep_col[k];
            emap[base + e * 32 + t] = d.dep_src[k];
          }
        }
        slice_ent.push_back(base);
        slice_len.push_back(len);
      }
      for (int r : longrows) {
        slice_ent.push_back((int)ecol.size());
        slice_len.push_back(-deps_of(r));
        for (int k = d.row_ptr[r]; k < d.row_ptr[r + 1]; ++k) {
          ecol.push_back(d.dep_col[k]);
          emap.push_back(d.dep_src[k]);
        }
        slice_rows.push_back(r);
        dmap.push_back(d.diag_src[r]);
        for (int t = 1; t < 32; ++t) {
          slice_rows.push_back(-1);
          dmap.push_back(-1);
        }
      }
      lvl_slice.push_back((int)slice_len.size());
    }
    tile_lvl.push_back((int)lvl_slice.size() - 1);
  }
  plan->n = n;
  plan->lower = lower;
  plan->nlevels = nlev;
  plan->tile_rows = tile_rows;
  plan->ntiles = ntiles;
  plan->nlvl = (int)lvl_slice.size() - 1;
  plan->nslices = (int)slice_len.size();
  plan->nent = (int)ecol.size();
  plan->ndeps = (long long)d.dep_col.size();
  plan->norder = (int)order.size();
  GB_TRY(upload(&plan->tile_row0, tr0));
  GB_TRY(upload(&plan->tile_row1, tr1));
  GB_TRY(upload(&plan->tile_lvl, tile_lvl));
  GB_TRY(upload(&plan->lvl_slice, lvl_slice));
  GB_TRY(upload(&plan->slice_rows, slice_rows));
  GB_TRY(upload(&plan->slice_ent, slice_ent));
  GB_TRY(upload(&plan->slice_len, slice_len));
  GB_TRY(upload(&plan->ecol, ecol));
  GB_TRY(upload(&plan->emap, emap));
  GB_TRY(upload(&plan->dmap, dmap));
  GB_TRY(upload(&plan->order, order));
  GB_CUDA_TRY(cudaMalloc(&plan->eval, sizeof(double) * std::max(1, plan->nent)));
  GB_CUDA_TRY(cudaMalloc(&plan->diag, sizeof(double) * std::max(1, plan->nslices * 32)));
  GB_CUDA_TRY(cudaMalloc(&plan->dinv, sizeof(double) * std::max(1, plan->nslices * 32)));
  GB_CUDA_TRY(cudaMalloc(&plan->ticket, sizeof(unsigned) * 4));
  GB_CUDA_TRY(cudaMemset(plan->ticket, 0, sizeof(unsigned) * 4));
  return GB_OK;
}

void tri_plan_free(TriPlan* p) {
  void* ptrs[] = {p->tile_row0, p->tile_row1, p->tile_lvl, p->lvl_slice, p->slice_rows,
                  p->slice_ent, p->slice_len, p->ecol,     p->emap,      p->dmap,
                  p->eval,      p->diag,      p->dinv,     p->eval32,    p->diag32,
                  p->dinv32,    p->order,     p->ticket};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  *p = TriPlan();
}

__global__ void recip_kernel(int n, const double* __restrict__ d, double* r, float* r32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = d[i] != 0.0 ? 1.0 / d[i] : 0.0;
    r[i] = v;
    if (r32) r32[i] = (float)v;
  }
}

int tri_plan_fill(TriPlan* p, const double* ent_src, const double* diag_src, bool want32,
                  cudaStream_t s) {
  const int nd = p->nslices * 32;
  if (want32 && !p->eval32) {
    GB_CUDA_TRY(cudaMalloc(&p->eval32, sizeof(float) * std::max(1, p->nent)));
    GB_CUDA_TRY(cudaMalloc(&p->diag32, sizeof(float) * std::max(1, nd)));
    GB_CUDA_TRY(cudaMalloc(&p->dinv32, sizeof(float) * std::max(1, nd)));
  }
  GB_TRY(gather_values(p->nent, p->emap, ent_src, p->eval, want32 ? p->eval32 : nullptr, s));
  GB_TRY(gather_values(nd, p->dmap, diag_src, p->diag, want32 ? p->diag32 : nullptr, s));
  if (nd > 0) {
    recip_kernel<<<std::max(1, std::min(device_sm_count() * 8, ceil_div(nd, 256))), 256, 0, s>>>(
        nd, p->diag, p->dinv, want32 ? p->dinv32 : nullptr);
    GB_CUDA_TRY(cudaGetLastError());
  }
  return GB_OK;
}

// ------------------------------------------------------------ launching
static int g_tri_bps = 0;

int tri_blocks_per_sm() {
  if (g_tri_bps == 0) {
    const char* e = getenv("GBLAP_TRI_BLOCKS_PER_SM");
    const int v = e ? atoi(e) : 0;
    g_tri_bps = (v >= 1 && v <= 8) ? v : 1;
  }
  return g_tri_bps;
}

void tri_set_blocks_per_sm(int bps) { g_tri_bps = std::max(1, std::min(8, bps)); }

int tri_grid(int ntiles) {
  return std::max(1, std::min(ntiles, device_sm_count() * tri_blocks_per_sm()));
}

template <typename T>
TriArgs<T> tri_args(const TriPlan& p, T* y, int* err) {
  TriArgs<T> A;
  A.ntiles = p.ntiles;
  A.tile_row0 = p.tile_row0;
  A.tile_row1 = p.tile_row1;
  A.tile_lvl = p.tile_lvl;
  A.lvl_slice = p.lvl_slice;
  A.slice_rows = p.slice_rows;
  A.slice_ent = p.slice_ent;
  A.slice_len = p.slice_len;
  A.ecol = p.ecol;
  if constexpr (sizeof(T) == 8) {
    A.eval = (const T*)p.eval;
    A.diag = (const T*)p.diag;
    A.dinv = (const T*)p.dinv;
  } else {
    A.eval = (const T*)p.eval32;
    A.diag = (const T*)p.diag32;
    A.dinv = (const T*)p.dinv32;
  }
  A.y = y;
  A.ticket = p.ticket;
  A.err = err;
  A.lower = p.lower ? 1 : 0;
  return A;
}
template TriArgs<double> tri_args<double>(const TriPlan&, double*, int*);
template TriArgs<float> tri_args<float>(const TriPlan&, float*, int*);

template <typename T>
int tri_solve_plain(const TriPlan* p, const T* x, T* y, int* err, cudaStream_t s) {
  if (p->n <= 0) return GB_OK;
  GB_TRY(fill_sentinel_dev(p->n, y, s));
  OpPlain<T> op{x};
  return tri_launch<T, OpPlain<T>, true>(*p, tri_args<T>(*p, y, err), op, s);
}
template int tri_solve_plain<double>(const TriPlan*, const double*, double*, int*, cudaStream_t);
template int tri_solve_plain<float>(const TriPlan*, const float*, float*, int*, cudaStream_t);

// ------------------------------------------------------------ IC(0) factor
// Left-looking restatement of simple_blas.c:139-168: row j receives, for
// every i < j with (i, j) in the pattern and in increasing i, the update
// a_jc -= u_ij * u_ic for each c >= j shared by rows i and j -- exactly the
// updates, in exactly the order, that the reference's right-looking sweep
// applies to row j -- then u_jj = sqrt(a_jj) and u_jc = a_jc / u_jj.  Rows
// run in global level order (each level padded to whole warps, so a warp
// never waits on itself), taken in chunks by ticket; row j waits for its
// dependencies' done flags (acquire) and publishes its own (release).
__global__ void __launch_bounds__(256)
    ichol_factor_kernel(int norder, const int* __restrict__ order, const int* __restrict__ ia,
                        const int* __restrict__ ja, const int* __restrict__ dpos,
                        const int* __restrict__ tpos, double* f, int* done, unsigned* ticket,
                        int* zero_pivot, int* err) {
  __shared__ int s_chunk;
  const int nchunks = ceil_div(norder, 256);
  while (true) {
    if (threadIdx.x == 0) s_chunk = (int)atomicAdd(&ticket[0], 1u);
    __syncthreads();
    const int chunk = s_chunk;
    __syncthreads();
    if (chunk >= nchunks) break;
    const int slot = chunk * 256 + threadIdx.x;
    const int j = slot < norder ? order[slot] : -1;
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
  const int blocks = std::max(1, std::min(ceil_div(lp->norder, 256), device_sm_count() * 2));
  ichol_factor_kernel<<<blocks, 256, 0, s>>>(lp->norder, lp->order, ia, ja, dpos, tpos, f, done,
                                             ticket, zero_pivot, err);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
