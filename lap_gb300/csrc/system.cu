// system.cu -- gb_system: setup (validation, SpMV plan, level schedules,
// on-device IC(0)), the solve drivers (CUDA-graph while loop or eager), the
// FP32-inner / FP64-refinement solve, and the kernel-level entry points.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <chrono>
#include <thread>
#include <cstdio>
#include <vector>

#include "gb_common.cuh"
#include "kernels.h"
#include "pcg.h"
#include "pcg_state.cuh"
#include "sptrsv.h"
#include "system.h"

using namespace gb;

// ------------------------------------------------------------ names / status
extern "C" const char* gb_status_str(int s) {
  switch (s) {
    case GB_OK: return "ok";
    case GB_MAXIT: return "maximum iterations reached";
    case GB_BREAKDOWN: return "breakdown (p'q <= 0 or non-finite)";
    case GB_ZERO_PIVOT: return "IC(0) zero or negative pivot";
    case GB_TIMEOUT: return "sync-free wait timed out";
    case GB_BAD_INPUT: return "bad input";
    case GB_CUDA_ERROR: return "CUDA error";
    case GB_NO_MEMORY: return "out of device memory";
    case GB_NOT_SUPPORTED: return "not supported";
    case GB_INTERNAL: return "device-side consistency check failed";
  }
  return "unknown status";
}

extern "C" int gb_prec_from_name(const char* name) {
  if (!name) return -1;
  static const char* names[] = {"none", "line_jacobi", "it_jacobi", "GS_std", "GS_it", "GS_it2", "ichol"};
  for (int i = 0; i < 7; ++i)
    if (strcmp(name, names[i]) == 0) return i;
  return -1;
}

extern "C" const char* gb_version(void) { return "libgblap 0.1 (sm_103a, CUDA " GB_STR(__CUDACC_VER_MAJOR__) ")"; }

extern "C" void gb_pcg_opts_default(gb_pcg_opts* o) {
  if (!o) return;
  o->tol = 1e-8;
  o->maxit = 10000;
  o->precision = 0;
  o->inner_tol = 0.0;  // the mode's default
  o->max_outer = 50;
  o->use_graph = 1;
  o->verbose = 0;
}

// ------------------------------------------------------------ helpers
namespace {

template <typename V>
int dalloc(V** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, sizeof(V) * std::max<size_t>(count, 1));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return e == cudaErrorMemoryAllocation ? GB_NO_MEMORY : GB_CUDA_ERROR;
  }
  return GB_OK;
}
template <typename V>
int dupload(V** p, const std::vector<V>& h) {
  GB_TRY(dalloc(p, h.size()));
  if (!h.empty()) GB_CUDA_TRY(cudaMemcpy(*p, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice));
  return GB_OK;
}

// Full symmetric CSR -> strict one-sided dependency list, diagonal from A.
int deps_from_full(int n, const int* ia, const int* ja, const std::vector<int>& dpos, bool lower,
                   TriDeps* d) {
  d->n = n;
  d->lower = lower;
  d->row_ptr.assign(n + 1, 0);
  d->diag_src = dpos;
  d->dep_col.clear();
  d->dep_src.clear();
  for (int i = 0; i < n; ++i) {
    for (int k = ia[i]; k < ia[i + 1]; ++k) {
      const int c = ja[k];
      if ((lower && c < i) || (!lower && c > i)) {
        d->dep_col.push_back(c);
        d->dep_src.push_back(k);
      }
    }
    d->row_ptr[i + 1] = (int)d->dep_col.size();
  }
  return GB_OK;
}

void init_state_host(PcgState* h, double tol, int maxit, int hist_len) {
  memset(h, 0, sizeof(*h));
  h->spare0 = tol;
  h->maxit = maxit;
  h->hist_len = hist_len;
  h->flag = 1;
  h->status = GB_OK;
}

}  // namespace

namespace gb {
int system_ensure_hist(gb_system sys, int maxit) {
  const int need = maxit + 3;
  if (sys->hist_cap >= need) return GB_OK;
  if (sys->hist) cudaFree(sys->hist);
  sys->hist = nullptr;
  GB_TRY(dalloc(&sys->hist, need));
  sys->hist_cap = need;
  for (auto& lg : sys->loop) {  // graphs captured the old pointer
    if (lg.exec) cudaGraphExecDestroy(lg.exec);
    if (lg.graph) cudaGraphDestroy(lg.graph);
    lg = LoopGraph();
  }
  sys->loop_key[0] = sys->loop_key[1] = -1;
  return GB_OK;
}
}  // namespace gb

static void system_free(gb_system s) {
  if (!s) return;
  for (auto& lg : s->loop) {
    if (lg.exec) cudaGraphExecDestroy(lg.exec);
    if (lg.graph) cudaGraphDestroy(lg.graph);
  }
  batch_release(s->multi);
  s->multi = nullptr;
  batch_release(s->multi_tail);
  s->multi_tail = nullptr;
  spmv_plan_free(&s->plan);
  tri_plan_free(&s->L);
  tri_plan_free(&s->U);
  tri_plan_free(&s->L32);
  tri_plan_free(&s->U32);
  void* ptrs[] = {s->dpos, s->tpos, s->diag, s->d_r, s->d_r32, s->a32, s->fac, s->fac_done,
                  s->zero_pivot, s->fac_ticket, s->lia, s->lja, s->uia, s->uja, s->la, s->ua,
                  s->v64.x, s->v64.r, s->v64.w, s->v64.p0, s->v64.p1, s->v64.q, s->v64.t,
                  s->v64.s, s->v32.x, s->v32.r, s->v32.w, s->v32.p0, s->v32.p1, s->v32.q,
                  s->v32.t, s->v32.s, s->b_int, s->aux1, s->aux2, s->aux3, s->part, s->st,
                  s->st_out, s->hist, s->err, s->lower_idx, s->lower_row, s->lmap_cpu,
                  s->umap_cpu, s->scratch, s->edge_idx, s->edge_row, s->pv_l, s->pv_u, s->hash_dev};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (s->st_host) cudaFreeHost(s->st_host);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->s) cudaStreamDestroy(s->s);
  delete s;
}

// Validates a full symmetric CSR (0-based, sorted, no duplicates, diagonal
// stored).  LAP itself does not check (io_utils.c:141-363 trusts its input;
// a missing diagonal corrupts memory in split()).
static int validate_csr(int n, int nnz, const std::vector<int>& ia, const std::vector<int>& ja,
                        std::vector<int>* dpos) {
  if (ia[0] != 0 || ia[n] != nnz) return GB_BAD_INPUT;
  dpos->assign(n, -1);
  for (int i = 0; i < n; ++i) {
    if (ia[i + 1] < ia[i]) return GB_BAD_INPUT;
    int prev = -1;
    for (int k = ia[i]; k < ia[i + 1]; ++k) {
      const int c = ja[k];
      if (c < 0 || c >= n || c <= prev) return GB_BAD_INPUT;
      prev = c;
      if (c == i) (*dpos)[i] = k;
    }
    if ((*dpos)[i] < 0) return GB_BAD_INPUT;
  }
  return GB_OK;
}

// A's derived arrays: diagonal, its reciprocal (FP64, FP32), FP32 values.
static int setup_matrix_values(gb_system s) {
  const int n = s->n;
  GB_TRY(gather_values(n, s->dpos, s->a, s->diag, nullptr, s->s));
  GB_TRY(reciprocal_dev(n, s->diag, s->d_r, s->s));
  GB_TRY(cast_f64_to_f32(n, s->d_r, s->d_r32, s->s));
  GB_TRY(cast_f64_to_f32(s->nnz, s->a, s->a32, s->s));
  return GB_OK;
}

static int setup_values(gb_system s) {
  const int n = s->n;
  GB_TRY(setup_matrix_values(s));
  if (s->prec == GB_PREC_GS_STD) {
    GB_TRY(tri_plan_fill(&s->L, s->a, s->a, kFillFma64, s->s));
    GB_TRY(tri_plan_fill(&s->U, s->a, s->a, kFillFma64, s->s));
    GB_TRY(tri_plan_fill(&s->L32, s->a, s->a, kFillFma32, s->s));
    GB_TRY(tri_plan_fill(&s->U32, s->a, s->a, kFillFma32, s->s));
  } else if (s->prec == GB_PREC_ICHOL) {
    GB_TRY(ichol_factor_dev(n, s->ia, s->ja, s->a, s->dpos, s->tpos, &s->L, s->fac, s->fac_done,
                            s->fac_ticket, s->zero_pivot, s->err, s->s));
    GB_TRY(tri_plan_fill(&s->L, s->fac, s->fac, kFillFma64, s->s));
    GB_TRY(tri_plan_fill(&s->U, s->fac, s->fac, kFillFma64, s->s));
    GB_TRY(tri_plan_fill(&s->L32, s->fac, s->fac, kFillFma32, s->s));
    GB_TRY(tri_plan_fill(&s->U32, s->fac, s->fac, kFillFma32, s->s));
  } else if (s->prec == GB_PREC_IT_JACOBI || s->prec == GB_PREC_GS_IT || s->prec == GB_PREC_GS_IT2) {
    GB_TRY(gather_values(s->lnnz, s->lmap_cpu, s->a, s->la, nullptr, s->s));
    GB_TRY(gather_values(s->unnz, s->umap_cpu, s->a, s->ua, nullptr, s->s));
  }
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  if (s->prec == GB_PREC_ICHOL) {
    int zp = 0, err = 0;
    GB_CUDA_TRY(cudaMemcpy(&zp, s->zero_pivot, sizeof(int), cudaMemcpyDeviceToHost));
    GB_CUDA_TRY(cudaMemcpy(&err, s->err, sizeof(int), cudaMemcpyDeviceToHost));
    s->zero_pivot_row = zp;
    if (err) return err;
  }
  return GB_OK;
}

namespace {
// Setup phase timer: GBLAP_VERBOSE=1 prints each phase's wall time to stderr.
struct PhaseTimer {
  bool on = false;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  PhaseTimer() {
    const char* v = getenv("GBLAP_VERBOSE");
    on = v && v[0] && v[0] != '0';
  }
  void mark(const char* what) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    fprintf(stderr, "libgblap: setup %-28s %9.1f ms\n", what,
            std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};
}  // namespace

extern "C" int gb_system_create(int n, int nnz, const int* ia, const int* ja, const double* a,
                                const char* prec_name, int m, int k, gb_system* out) {
  PhaseTimer ph;
  if (!out) return GB_BAD_INPUT;
  *out = nullptr;
  const int prec = gb_prec_from_name(prec_name);
  if (n <= 0 || nnz < n || !ia || !ja || !a || prec < 0 || m < 0 || k < 0) return GB_BAD_INPUT;
  gb_system s = new gb_system_s();
  s->n = n;
  s->nnz = nnz;
  s->ia = ia;
  s->ja = ja;
  s->a = a;
  s->prec = prec;
  s->m = m;
  s->k = k;
  int rc = GB_OK;
#define CK(expr)            \
  do {                      \
    rc = (expr);            \
    if (rc != GB_OK) {      \
      system_free(s);       \
      return rc;            \
    }                       \
  } while (0)
#define CKC(expr) CK((expr) == cudaSuccess ? GB_OK : GB_CUDA_ERROR)
  CKC(cudaStreamCreateWithFlags(&s->s, cudaStreamNonBlocking));
  CKC(cudaEventCreate(&s->ev0));
  CKC(cudaEventCreate(&s->ev1));
  s->h_ia.resize(n + 1);
  s->h_ja.resize(nnz);
  CKC(cudaMemcpy(s->h_ia.data(), ia, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
  CKC(cudaMemcpy(s->h_ja.data(), ja, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToHost));
  std::vector<int> dpos;
  CK(validate_csr(n, nnz, s->h_ia, s->h_ja, &dpos));
  ph.mark("copy + validate");
  CK(spmv_plan_build(n, nnz, s->h_ia.data(), &s->plan, kBundleRows));
  CK(dupload(&s->dpos, dpos));
  CK(dalloc(&s->diag, n));
  CK(dalloc(&s->d_r, n));
  CK(dalloc(&s->d_r32, n));
  CK(dalloc(&s->a32, nnz));
  CK(dalloc(&s->err, 4));
  CKC(cudaMemset(s->err, 0, sizeof(int) * 4));
  const int* hia = s->h_ia.data();
  const int* hja = s->h_ja.data();
  std::vector<int> tpos;
  CK(transpose_positions(n, hia, hja, &tpos));  // also proves the pattern symmetric
  ph.mark("spmv plan + transpose");
  CK(dupload(&s->tpos, tpos));
  if (prec == GB_PREC_GS_STD || prec == GB_PREC_ICHOL) {
    s->tri = true;
    TriDeps dl, du;
    if (prec == GB_PREC_GS_STD) {
      CK(deps_from_full(n, hia, hja, dpos, true, &dl));
      CK(deps_from_full(n, hia, hja, dpos, false, &du));
    } else {
      CK(deps_ichol(n, hia, hja, tpos, true, &dl));
      CK(deps_ichol(n, hia, hja, tpos, false, &du));
      CK(dalloc(&s->fac, nnz));
      CK(dalloc(&s->fac_done, n));
      CK(dalloc(&s->zero_pivot, 1));
      CK(dalloc(&s->fac_ticket, 4));
      CKC(cudaMemset(s->fac_ticket, 0, sizeof(unsigned) * 4));
    }
    ph.mark("dependency lists");
    // FP32 tiles of both factors as tall as the FP64 ones, which leaves
    // shared memory for the inbox of the pushing cluster form; both FP32
    // solves poll values there (128^3 split solve: lower 284 vs 473 us on
    // twice-as-tall tiles in pulling clusters; upper 250 vs 267 us).
    // GBLAP_TRI_TILE_ROWS32 sets both explicitly.
    const int t32l = tri_default_tile_rows32(n);
    const int t32u = t32l;
    // The four plans are independent host work (levels, record packing,
    // layout): built on parallel threads, each with this thread's device
    // current (4.19M-row Chung-Lu: 8.8 s one after another).
    {
      int dev = 0;
      CKC(cudaGetDevice(&dev));
      (void)device_sm_count();  // initialised once here, read by the workers
      const int w32 = tri_consumer_warps(4);
      int rcs[4] = {GB_OK, GB_OK, GB_OK, GB_OK};
      std::thread th[4] = {
          std::thread([&] { rcs[0] = cudaSetDevice(dev) == cudaSuccess ? tri_plan_build(dl, &s->L) : GB_CUDA_ERROR; }),
          std::thread([&] { rcs[1] = cudaSetDevice(dev) == cudaSuccess ? tri_plan_build(du, &s->U) : GB_CUDA_ERROR; }),
          std::thread([&] {
            rcs[2] = cudaSetDevice(dev) == cudaSuccess ? tri_plan_build(dl, &s->L32, t32l, w32) : GB_CUDA_ERROR;
          }),
          std::thread([&] {
            rcs[3] = cudaSetDevice(dev) == cudaSuccess ? tri_plan_build(du, &s->U32, t32u, w32) : GB_CUDA_ERROR;
          })};
      for (auto& t : th) t.join();
      for (int r : rcs) CK(r);
    }
    ph.mark("triangular plans");
  }
  if (prec == GB_PREC_GS_STD) {
    // LAP's CUDA driver hands GS_std its L and U with the diagonal inside:
    // last in each L row, first in each U row (cg_driver2.c:95-144)
    std::vector<int> lp(n + 1, 0), up(n + 1, 0), lj, uj;
    for (int i = 0; i < n; ++i) {
      for (int q = hia[i]; q < hia[i + 1]; ++q)
        if (hja[q] < i) lj.push_back(hja[q]);
      lj.push_back(i);
      uj.push_back(i);
      for (int q = hia[i]; q < hia[i + 1]; ++q)
        if (hja[q] > i) uj.push_back(hja[q]);
      lp[i + 1] = (int)lj.size();
      up[i + 1] = (int)uj.size();
    }
    s->pl_nnz = (int)lj.size();
    s->pu_nnz = (int)uj.size();
    s->pat_l = pattern_hash_host(n, s->pl_nnz, lp.data(), lj.data());
    s->pat_u = pattern_hash_host(n, s->pu_nnz, up.data(), uj.data());
  }
  if (prec == GB_PREC_IT_JACOBI || prec == GB_PREC_GS_IT || prec == GB_PREC_GS_IT2) {
    std::vector<int> lp(n + 1, 0), up(n + 1, 0), lj, uj, lm, um;
    for (int i = 0; i < n; ++i) {
      for (int q = hia[i]; q < hia[i + 1]; ++q) {
        if (hja[q] < i) { lj.push_back(hja[q]); lm.push_back(q); }
        if (hja[q] > i) { uj.push_back(hja[q]); um.push_back(q); }
      }
      lp[i + 1] = (int)lj.size();
      up[i + 1] = (int)uj.size();
    }
    s->lnnz = (int)lj.size();
    s->unnz = (int)uj.size();
    s->pl_nnz = s->lnnz;
    s->pu_nnz = s->unnz;
    s->pat_l = pattern_hash_host(n, s->lnnz, lp.data(), lj.data());
    s->pat_u = pattern_hash_host(n, s->unnz, up.data(), uj.data());
    CK(dupload(&s->lia, lp));
    CK(dupload(&s->uia, up));
    CK(dupload(&s->lja, lj));
    CK(dupload(&s->uja, uj));
    CK(dupload(&s->lmap_cpu, lm));
    CK(dupload(&s->umap_cpu, um));
    CK(dalloc(&s->la, s->lnnz));
    CK(dalloc(&s->ua, s->unnz));
  }
  ph.mark("other maps");
  // work vectors
  for (double** p : {&s->v64.x, &s->v64.r, &s->v64.w, &s->v64.p0, &s->v64.p1, &s->v64.q,
                     &s->v64.t, &s->v64.s, &s->b_int, &s->aux1, &s->aux2, &s->aux3})
    CK(dalloc(p, n));
  for (float** p : {&s->v32.x, &s->v32.r, &s->v32.w, &s->v32.p0, &s->v32.p1, &s->v32.q,
                    &s->v32.t, &s->v32.s})
    CK(dalloc(p, n));
  s->part_len = part_len_needed(s);
  CK(dalloc(&s->part, s->part_len));
  CK(dalloc(&s->st, 1));
  CK(dalloc(&s->st_out, 1));
  CK(dalloc(&s->scratch, 8));
  CK(dalloc(&s->hash_dev, 1));
  CKC(cudaMemset(s->st, 0, sizeof(PcgState)));
  CKC(cudaMemset(s->st_out, 0, sizeof(PcgState)));
  CKC(cudaMallocHost(&s->st_host, sizeof(PcgState) * 2));
  CK(system_ensure_hist(s, 1000));
  ph.mark("buffers");
  CK(setup_values(s));
  ph.mark("values (IC(0) factor, fills)");
#undef CK
#undef CKC
  *out = s;
  return GB_OK;
}

extern "C" int gb_system_destroy(gb_system s) {
  if (!s) return GB_BAD_INPUT;
  cudaStreamSynchronize(s->s);
  system_free(s);
  return GB_OK;
}

extern "C" int gb_debug_set_spin_budget(gb_system s, unsigned long long ns) {
  if (!s) return GB_BAD_INPUT;
  GB_CUDA_TRY(cudaMemcpy(s->err + 2, &ns, sizeof ns, cudaMemcpyHostToDevice));
  return GB_OK;
}

extern "C" int gb_system_update_values(gb_system s) {
  if (!s) return GB_BAD_INPUT;
  return setup_values(s);
}

extern "C" int gb_system_refresh_matrix(gb_system s) {
  if (!s) return GB_BAD_INPUT;
  GB_TRY(setup_matrix_values(s));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  return GB_OK;
}

extern "C" int gb_system_pattern_hash(gb_system s, int n, int nnz, const int* ia, const int* ja,
                                      unsigned long long* out) {
  if (!s || !out) return GB_BAD_INPUT;
  return pattern_hash(n, nnz, ia, ja, s->hash_dev, s->s, out);
}

namespace {
// GS_std's L (diagonal last) and U (diagonal first) onto A's pattern: row i's
// L entries are A's entries ia[i] .. dpos[i], its U entries dpos[i] .. ia[i+1]-1
// (the layouts were checked against the system's before this runs).
__global__ void scatter_embedded_kernel(int n, const int* __restrict__ ia, const int* __restrict__ dpos,
                                        const int* __restrict__ lia, const double* __restrict__ la,
                                        const int* __restrict__ uia, const double* __restrict__ ua,
                                        double* pv_l, double* pv_u) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int a0 = ia[i], d = dpos[i], a1 = ia[i + 1], l0 = lia[i], u0 = uia[i];
    for (int t = 0; t <= d - a0; ++t) pv_l[a0 + t] = la[l0 + t];
    for (int t = 0; t < a1 - d; ++t) pv_u[d + t] = ua[u0 + t];
  }
}
}  // namespace

extern "C" int gb_system_set_prec_values(gb_system s, const int* lia, const int* lja, const double* la,
                                         int lnnz, const int* uia, const int* uja, const double* ua,
                                         int unnz, const double* d_r, const double* ichol_vals) {
  if (!s) return GB_BAD_INPUT;
  const int n = s->n;
  auto check_lu = [&]() -> int {
    if (!lia || !lja || !la || !uia || !uja || !ua) return GB_BAD_INPUT;
    if (lnnz != s->pl_nnz || unnz != s->pu_nnz) return GB_BAD_INPUT;
    unsigned long long hl = 0, hu = 0;
    GB_TRY(pattern_hash(n, lnnz, lia, lja, s->hash_dev, s->s, &hl));
    GB_TRY(pattern_hash(n, unnz, uia, uja, s->hash_dev, s->s, &hu));
    return (hl == s->pat_l && hu == s->pat_u) ? GB_OK : GB_BAD_INPUT;
  };
  auto load_d_r = [&]() -> int {
    if (!d_r) return GB_BAD_INPUT;
    GB_TRY(copy_dev(n, d_r, s->d_r, s->s));
    return cast_f64_to_f32(n, s->d_r, s->d_r32, s->s);
  };
  switch (s->prec) {
    case GB_PREC_NONE:
      break;
    case GB_PREC_LINE_JACOBI:
      GB_TRY(load_d_r());
      break;
    case GB_PREC_IT_JACOBI:
    case GB_PREC_GS_IT:
    case GB_PREC_GS_IT2:
      GB_TRY(check_lu());
      GB_TRY(load_d_r());
      GB_TRY(copy_dev(lnnz, la, s->la, s->s));
      GB_TRY(copy_dev(unnz, ua, s->ua, s->s));
      break;
    case GB_PREC_GS_STD: {
      GB_TRY(check_lu());
      if (!s->pv_l) GB_TRY(dalloc(&s->pv_l, s->nnz));
      if (!s->pv_u) GB_TRY(dalloc(&s->pv_u, s->nnz));
      const int grid = std::max(1, std::min((n + 255) / 256, reduction_grid()));
      scatter_embedded_kernel<<<grid, 256, 0, s->s>>>(n, s->ia, s->dpos, lia, la, uia, ua, s->pv_l, s->pv_u);
      GB_CUDA_TRY(cudaGetLastError());
      GB_TRY(tri_plan_fill(&s->L, s->pv_l, s->pv_l, kFillFma64, s->s));
      GB_TRY(tri_plan_fill(&s->U, s->pv_u, s->pv_u, kFillFma64, s->s));
      GB_TRY(tri_plan_fill(&s->L32, s->pv_l, s->pv_l, kFillFma32, s->s));
      GB_TRY(tri_plan_fill(&s->U32, s->pv_u, s->pv_u, kFillFma32, s->s));
      break;
    }
    case GB_PREC_ICHOL:
      // the factor as initialize_ichol leaves it: L in A's lower triangle
      // (diagonal included); the upper solve reads L's entries transposed
      if (!ichol_vals) return GB_BAD_INPUT;
      GB_TRY(tri_plan_fill(&s->L, ichol_vals, ichol_vals, kFillFma64, s->s));
      GB_TRY(tri_plan_fill(&s->U, ichol_vals, ichol_vals, kFillFma64, s->s));
      GB_TRY(tri_plan_fill(&s->L32, ichol_vals, ichol_vals, kFillFma32, s->s));
      GB_TRY(tri_plan_fill(&s->U32, ichol_vals, ichol_vals, kFillFma32, s->s));
      s->zero_pivot_row = 0;
      break;
    default:
      return GB_BAD_INPUT;
  }
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  return GB_OK;
}

extern "C" int gb_system_info(gb_system s, int* lower_levels, int* upper_levels, int* tiles) {
  if (!s) return GB_BAD_INPUT;
  if (lower_levels) *lower_levels = s->L.nlevels;
  if (upper_levels) *upper_levels = s->U.nlevels;
  if (tiles) *tiles = s->plan.nbundles;
  return s->zero_pivot_row ? GB_ZERO_PIVOT : GB_OK;
}

// ------------------------------------------------------------ solve loop
// Builds (once) a graph holding only a while node whose body is one PCG
// iteration; the body's checking kernel sets the condition.
using BodyFn = int (*)(gb_system, PcgState*, cudaGraphConditionalHandle, int);

static int get_loop_graph(gb_system s, int idx, BodyFn body_fn, LoopGraph** out) {
  LoopGraph* lg = &s->loop[idx];
  const int key = s->hist_cap;
  if (lg->exec && s->loop_key[idx] == key) {
    *out = lg;
    return GB_OK;
  }
  if (lg->exec) cudaGraphExecDestroy(lg->exec);
  if (lg->graph) cudaGraphDestroy(lg->graph);
  *lg = LoopGraph();
  cudaGraph_t g;
  GB_CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  GB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  // cudaGraphNodeParams has no usable default constructor in C++; start from
  // zeroed storage as the C API expects
  alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
  memset(cp_buf, 0, sizeof cp_buf);
  cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cp_buf);
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  GB_CUDA_TRY(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  GB_CUDA_TRY(cudaStreamBeginCaptureToGraph(s->s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const int rc = body_fn(s, s->st, h, 1);
  cudaGraph_t captured = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s->s, &captured);
  if (rc != GB_OK || e != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    return rc != GB_OK ? rc : GB_CUDA_ERROR;
  }
  GB_CUDA_TRY(cudaGraphInstantiate(&lg->exec, g, 0));
  lg->graph = g;
  s->loop_key[idx] = key;
  *out = lg;
  return GB_OK;
}

// Runs one PCG recurrence on the system stream: prologue, then the loop.
static int run_loop(gb_system s, int idx, BodyFn body_fn, int maxit, int use_graph);

template <typename T>
static int run_recurrence(gb_system s, double tol, int maxit, int x_zero, const T* b, int use_graph) {
  init_state_host(s->st_host, tol, maxit, s->hist_cap);
  GB_CUDA_TRY(cudaMemcpyAsync(s->st, s->st_host, sizeof(PcgState), cudaMemcpyHostToDevice, s->s));
  GB_TRY(launch_prologue<T>(s, s->st, x_zero, b));
  return run_loop(s, sizeof(T) == 8 ? 0 : 1, &launch_body<T>, maxit, use_graph);
}

// Split precision: FP64 recurrence from x (not zeroed), FP32 operator and
// preconditioner.
static int run_recurrence_split(gb_system s, double tol, int maxit, const double* b, int use_graph) {
  init_state_host(s->st_host, tol, maxit, s->hist_cap);
  GB_CUDA_TRY(cudaMemcpyAsync(s->st, s->st_host, sizeof(PcgState), cudaMemcpyHostToDevice, s->s));
  GB_TRY(launch_prologue_split(s, s->st, b));
  return run_loop(s, 2, &launch_body_split, maxit, use_graph);
}

// Runs (or resumes) the iteration loop until the recurrence's done flag.
static int run_loop(gb_system s, int idx, BodyFn body_fn, int maxit, int use_graph) {
  if (use_graph) {
    LoopGraph* lg = nullptr;
    GB_TRY(get_loop_graph(s, idx, body_fn, &lg));
    GB_CUDA_TRY(cudaGraphLaunch(lg->exec, s->s));
  } else {
    // eager: a status read every 16 iterations
    for (int it = 0; it <= maxit + 1; it += 16) {
      for (int j = 0; j < 16; ++j) GB_TRY(body_fn(s, s->st, 0, 0));
      GB_CUDA_TRY(cudaMemcpyAsync(s->st_host, s->st, sizeof(PcgState), cudaMemcpyDeviceToHost, s->s));
      GB_CUDA_TRY(cudaStreamSynchronize(s->s));
      if (s->st_host->done) break;
    }
  }
  return GB_OK;
}

static int read_state(gb_system s, PcgState* dst, const PcgState* src) {
  GB_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(PcgState), cudaMemcpyDeviceToHost, s->s));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  return GB_OK;
}

// Core solve on the internal buffers b_int (rhs) and v64.x (x0 -> x).
static int solve_internal(gb_system s, const gb_pcg_opts* oin, gb_pcg_result* res, double* hist_host,
                          int hist_len) {
  gb_pcg_opts oc = *oin;
  if (oc.precision < 0) oc.precision = s->auto_precision;  // the autotuner's choice
  const gb_pcg_opts* o = &oc;
  GB_TRY(system_ensure_hist(s, o->maxit));
  GB_CUDA_TRY(cudaMemsetAsync(s->err, 0, sizeof(int), s->s));
  gb_pcg_result r;
  memset(&r, 0, sizeof r);
  PcgState* hs = s->st_host;
  // residual reduction between replacements: FP32 Krylov vectors (1) drift
  // slowly, the FP32 operator under FP64 vectors (2) is best replaced often
  const double itol = o->inner_tol > 0.0 ? o->inner_tol : (o->precision == 2 ? 1e-2 : 1e-4);
  if (o->precision == 0) {
    GB_TRY(run_recurrence<double>(s, o->tol, o->maxit, 0, s->b_int, o->use_graph));
    GB_TRY(launch_true_resid(s, s->b_int, s->v64.x, s->scratch));
    GB_TRY(read_state(s, hs, s->st));
    r.iters = hs->iter;
    r.flag = hs->flag;
    r.status = hs->status;
    r.res0 = hs->res0;
    r.res = std::sqrt(hs->rr);
    if (hist_host && hist_len > 0) {
      const int cnt = std::min(hist_len, std::min(hs->iter + 1, s->hist_cap));
      GB_CUDA_TRY(cudaMemcpy(hist_host, s->hist, sizeof(double) * cnt, cudaMemcpyDeviceToHost));
    }
  } else if (o->precision == 2) {
    if (!prec_fused_tri(s->prec, s->k)) return GB_NOT_SUPPORTED;
    PcgState* ho = s->st_host + 1;
    init_state_host(ho, o->tol, o->maxit, 0);
    GB_CUDA_TRY(cudaMemcpyAsync(s->st_out, ho, sizeof(PcgState), cudaMemcpyHostToDevice, s->s));
    // FP64 recurrence around the FP32 operator and preconditioner.  The
    // recursive residual drifts from b - A x by the FP32 rounding of A w that
    // q accumulates, so the recurrence pauses whenever its residual has
    // dropped by inner_tol since the last replacement; r is then replaced by
    // the FP64 true residual and the recurrence resumes with x, p, q and rho
    // intact.  Convergence is judged on the FP64 residual only.
    int total = 0, outer = 0, flag = 1, status = GB_MAXIT;
    GB_TRY(launch_outer_resid64(s, s->b_int, s->v64.x, 1));
    GB_TRY(read_state(s, ho, s->st_out));
    double last_res = std::sqrt(ho->rr);
    if (hist_host && hist_len > 0) hist_host[0] = last_res;
    if (ho->done) {
      flag = ho->flag;
      status = ho->status;
    } else {
      GB_TRY(run_recurrence_split(s, std::max(itol, o->tol), o->maxit, s->b_int, o->use_graph));
      for (;;) {
        GB_TRY(read_state(s, hs, s->st));
        total = hs->iter;
        if (hs->status == GB_BREAKDOWN) {
          flag = 2;
          status = GB_BREAKDOWN;
          break;
        }
        GB_TRY(launch_outer_resid64(s, s->b_int, s->v64.x, 0));
        GB_TRY(read_state(s, ho, s->st_out));
        ++outer;
        last_res = std::sqrt(ho->rr);
        if (hist_host && outer < hist_len) hist_host[outer] = last_res;
        if (ho->done) {
          flag = ho->flag;
          status = ho->status;
          break;
        }
        if (hs->flag == 1 || outer >= o->max_outer) break;  // out of iterations
        GB_TRY(launch_resume_split(s, s->st, itol));
        GB_TRY(run_loop(s, 2, &launch_body_split, o->maxit, o->use_graph));
      }
    }
    r.iters = total;
    r.outer = outer;
    r.flag = flag;
    r.status = status;
    r.res0 = ho->res0;
    r.res = last_res;
    GB_TRY(launch_true_resid(s, s->b_int, s->v64.x, s->scratch));
  } else if (o->precision == 1) {
    if (!(s->prec == GB_PREC_LINE_JACOBI || s->prec == GB_PREC_NONE || prec_fused_tri(s->prec, s->k)))
      return GB_NOT_SUPPORTED;
    PcgState* ho = s->st_host + 1;
    init_state_host(ho, o->tol, o->maxit, 0);
    GB_CUDA_TRY(cudaMemcpyAsync(s->st_out, ho, sizeof(PcgState), cudaMemcpyHostToDevice, s->s));
    // One FP32 PCG recurrence with residual replacement: it pauses whenever
    // its recursive residual has dropped by inner_tol since the last
    // replacement; the pause folds the FP32 correction into the FP64 x,
    // recomputes r = b - A x in FP64 (the refinement step), replaces the
    // FP32 residual with it and resumes with p, rho and the iteration count
    // intact -- no Krylov restart, so the iteration count stays close to the
    // FP64 PCG's.  Convergence is judged on the FP64 residual only.
    int total = 0, outer = 0, flag = 1, status = GB_MAXIT;
    double last_res = 0.0;
    GB_TRY(launch_outer_resid(s, s->b_int, s->v64.x, 1));
    GB_TRY(read_state(s, ho, s->st_out));
    last_res = std::sqrt(ho->rr);
    if (hist_host && hist_len > 0) hist_host[0] = last_res;
    if (ho->done) {
      flag = ho->flag;
      status = ho->status;
    } else {
      GB_TRY(run_recurrence<float>(s, std::max(itol, o->tol), o->maxit, 1, s->v32.r, o->use_graph));
      for (;;) {
        GB_TRY(read_state(s, hs, s->st));
        total = hs->iter;
        if (hs->status == GB_BREAKDOWN) {
          flag = 2;
          status = GB_BREAKDOWN;
          break;
        }
        GB_TRY(launch_add_correction(s, s->v64.x));
        GB_TRY(launch_outer_resid(s, s->b_int, s->v64.x, 0));  // also zeroes the FP32 x
        GB_TRY(read_state(s, ho, s->st_out));
        ++outer;
        last_res = std::sqrt(ho->rr);
        if (hist_host && outer < hist_len) hist_host[outer] = last_res;
        if (ho->done) {
          flag = ho->flag;
          status = ho->status;
          break;
        }
        if (hs->flag == 1 || outer >= o->max_outer) break;  // out of iterations
        GB_TRY(launch_resume<float>(s, s->st, itol));
        GB_TRY(run_loop(s, 1, &launch_body<float>, o->maxit, o->use_graph));
      }
    }
    r.iters = total;
    r.outer = outer;
    r.flag = flag;
    r.status = status;
    r.res0 = ho->res0;
    r.res = last_res;
    GB_TRY(launch_true_resid(s, s->b_int, s->v64.x, s->scratch));
  } else {
    return GB_BAD_INPUT;
  }
  double tr[2] = {0.0, 0.0};
  GB_CUDA_TRY(cudaMemcpyAsync(tr, s->scratch, sizeof tr, cudaMemcpyDeviceToHost, s->s));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  int err = 0;
  GB_CUDA_TRY(cudaMemcpy(&err, s->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) r.status = err;
  r.true_res = tr[0];
  r.rel_true_res = tr[1] > 0.0 ? tr[0] / tr[1] : tr[0];
  if (o->verbose && hist_host)
    for (int i = 0; i <= std::min(r.iters, hist_len - 1); ++i)
      printf("CG: it %d, res norm %5.5e \n", i, hist_host[i]);
  if (res) *res = r;
  return (r.status == GB_TIMEOUT || r.status == GB_INTERNAL) ? r.status : GB_OK;
}

extern "C" int gb_pcg_solve(gb_system s, const double* b, double* x, const gb_pcg_opts* opts,
                            double* hist_host, int hist_len, gb_pcg_result* res) {
  if (!s || !b || !x) return GB_BAD_INPUT;
  gb_pcg_opts o;
  if (opts) o = *opts;
  else gb_pcg_opts_default(&o);
  if (o.maxit < 0 || !(o.tol >= 0.0)) return GB_BAD_INPUT;
  const size_t bytes = sizeof(double) * s->n;
  GB_CUDA_TRY(cudaEventRecord(s->ev0, s->s));
  GB_CUDA_TRY(cudaMemcpyAsync(s->b_int, b, bytes, cudaMemcpyDeviceToDevice, s->s));
  GB_CUDA_TRY(cudaMemcpyAsync(s->v64.x, x, bytes, cudaMemcpyDeviceToDevice, s->s));
  const int rc = solve_internal(s, &o, res, hist_host, hist_len);
  GB_CUDA_TRY(cudaMemcpyAsync(x, s->v64.x, bytes, cudaMemcpyDeviceToDevice, s->s));
  GB_CUDA_TRY(cudaEventRecord(s->ev1, s->s));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s->ev0, s->ev1);
  if (res) res->device_ms = ms;
  return rc;
}

extern "C" int gb_pcg_solve_host(gb_system s, const double* b_host, double* x_host,
                                 const gb_pcg_opts* opts, gb_pcg_result* res) {
  if (!s || !b_host || !x_host) return GB_BAD_INPUT;
  gb_pcg_opts o;
  if (opts) o = *opts;
  else gb_pcg_opts_default(&o);
  const size_t bytes = sizeof(double) * s->n;
  GB_CUDA_TRY(cudaEventRecord(s->ev0, s->s));
  GB_CUDA_TRY(cudaMemcpyAsync(s->b_int, b_host, bytes, cudaMemcpyHostToDevice, s->s));
  GB_CUDA_TRY(cudaMemcpyAsync(s->v64.x, x_host, bytes, cudaMemcpyHostToDevice, s->s));
  const int rc = solve_internal(s, &o, res, nullptr, 0);
  GB_CUDA_TRY(cudaMemcpyAsync(x_host, s->v64.x, bytes, cudaMemcpyDeviceToHost, s->s));
  GB_CUDA_TRY(cudaEventRecord(s->ev1, s->s));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s->ev0, s->ev1);
  if (res) res->device_ms = ms;
  return rc;
}

// ------------------------------------------------------------ kernels
extern "C" int gb_spmv(gb_system s, double alpha, const double* x, double beta, double* y) {
  if (!s || !x || !y) return GB_BAD_INPUT;
  GB_TRY(spmv_axpby<double>(&s->plan, s->n, s->ia, s->ja, s->a, alpha, x, beta, y, s->s));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  return GB_OK;
}

extern "C" int gb_precond_apply(gb_system s, const double* x, double* y) {
  if (!s || !x || !y || x == y) return GB_BAD_INPUT;
  GB_CUDA_TRY(cudaMemsetAsync(s->err, 0, sizeof(int), s->s));
  GB_TRY(apply_prec(s, x, y));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  int err = 0;
  GB_CUDA_TRY(cudaMemcpy(&err, s->err, sizeof(int), cudaMemcpyDeviceToHost));
  return err ? err : GB_OK;
}

extern "C" int gb_ichol_factor_values(gb_system s, double* l_vals, double* u_vals) {
  if (!s || s->prec != GB_PREC_ICHOL) return GB_BAD_INPUT;
  // LAP CPU layout: L rows = strict lower entries then the diagonal; U rows =
  // diagonal then strict upper entries (cg_driver2.c:146-196).
  if (!s->lower_idx) {
    const int n = s->n;
    const int* hia = s->h_ia.data();
    const int* hja = s->h_ja.data();
    std::vector<int> lm, um;
    for (int i = 0; i < n; ++i) {
      int d = -1;
      for (int q = hia[i]; q < hia[i + 1]; ++q) {
        if (hja[q] < i) lm.push_back(q);
        if (hja[q] == i) d = q;
      }
      lm.push_back(d);
      um.push_back(d);
      for (int q = hia[i]; q < hia[i + 1]; ++q)
        if (hja[q] > i) um.push_back(q);
    }
    s->lu_len = (int)lm.size();
    GB_TRY(dupload(&s->lower_idx, lm));
    GB_TRY(dupload(&s->lower_row, um));
  }
  if (l_vals) GB_TRY(gather_values(s->lu_len, s->lower_idx, s->fac, l_vals, nullptr, s->s));
  if (u_vals) GB_TRY(gather_values(s->lu_len, s->lower_row, s->fac, u_vals, nullptr, s->s));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  return s->zero_pivot_row ? GB_ZERO_PIVOT : GB_OK;
}

extern "C" int gb_pcg_autotune_precision(gb_system s, const double* b, const gb_pcg_opts* opts, int* best,
                                         double* ms_host) {
  if (!s || !b) return GB_BAD_INPUT;
  gb_pcg_opts o;
  if (opts) o = *opts;
  else gb_pcg_opts_default(&o);
  double* x = nullptr;
  GB_CUDA_TRY(cudaMalloc(&x, sizeof(double) * s->n));
  int pick = -1, rc = GB_OK;
  double pick_ms = 0.0;
  for (int p = 0; p < 3 && rc == GB_OK; ++p) {
    o.precision = p;
    double t = -1.0;
    for (int rep = 0; rep < 2; ++rep) {
      if (cudaMemsetAsync(x, 0, sizeof(double) * s->n, s->s) != cudaSuccess) {
        rc = GB_CUDA_ERROR;
        break;
      }
      gb_pcg_result r;
      const int st = gb_pcg_solve(s, b, x, &o, nullptr, 0, &r);
      if (st == GB_NOT_SUPPORTED) {  // a mode this preconditioner has not
        t = -1.0;
        break;
      }
      if (st != GB_OK) {
        rc = st;
        break;
      }
      t = (r.status == GB_OK && r.flag == 0) ? r.device_ms : -1.0;
      if (t < 0.0) break;  // did not converge
    }
    if (ms_host) ms_host[p] = t;
    if (t >= 0.0 && (pick < 0 || t < pick_ms)) {
      pick = p;
      pick_ms = t;
    }
  }
  cudaFree(x);
  if (rc != GB_OK) return rc;
  if (pick < 0) return GB_MAXIT;
  s->auto_precision = pick;
  if (best) *best = pick;
  return GB_OK;
}
