// extras.cu -- adjoint gradient, SpMV autotuner and per-kernel profiling.
//
// None of these exists in LAP.  The adjoint reuses the same PCG on the
// adjoint right-hand side (A is SPD, so A^T = A) and adds one scatter kernel
// for dL/dA on A's pattern and dL/dw per edge.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "gb_common.cuh"
#include "kernels.h"
#include "pcg.h"
#include "pcg_state.cuh"
#include "system.h"

using namespace gb;

namespace {

// G[k] = -lambda_i * x_j for every stored entry k = (i, j): one warp per 32
// rows, lanes strided over the rows' contiguous entries (coalesced ja / G),
// the row of an entry found by bisection over the 33 row pointers.
__global__ void adjoint_scatter_kernel(int n, const int* __restrict__ ia, const int* __restrict__ ja,
                                       const double* __restrict__ x,
                                       const double* __restrict__ lambda, double* G) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 32 < n; w += nwarps) {
    const int r0 = w * 32;
    const int rows = min(32, n - r0);
    const int j0 = ia[r0];
    const int j1 = ia[r0 + rows];
    for (int j = j0 + lane; j < j1; j += 32) {
      int lo = 0, hi = rows - 1;
      while (lo < hi) {  // first row whose end > j
        const int mid = (lo + hi) >> 1;
        if (ia[r0 + mid + 1] > j) hi = mid;
        else lo = mid + 1;
      }
      const int i = r0 + lo;
      G[j] = -lambda[i] * x[ja[j]];
    }
  }
}

// dL/dw for every strict-lower entry (i, j) of A, row-major:
// -(lambda_i - lambda_j)(x_i - x_j) = G_ij + G_ji - G_ii - G_jj.
__global__ void edge_grad_kernel(int ne, const int* __restrict__ edge_idx,
                                 const int* __restrict__ edge_row, const int* __restrict__ ja,
                                 const double* __restrict__ x, const double* __restrict__ lambda,
                                 double* eg) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ne; t += gridDim.x * blockDim.x) {
    const int i = edge_row[t], j = ja[edge_idx[t]];
    eg[t] = -(lambda[i] - lambda[j]) * (x[i] - x[j]);
  }
}

int ensure_edges(gb_system s) {
  if (s->edge_idx) return GB_OK;
  std::vector<int> idx, row;
  for (int i = 0; i < s->n; ++i)
    for (int k = s->h_ia[i]; k < s->h_ia[i + 1]; ++k)
      if (s->h_ja[k] < i) {
        idx.push_back(k);
        row.push_back(i);
      }
  s->nedges = (int)idx.size();
  GB_CUDA_TRY(cudaMalloc(&s->edge_idx, sizeof(int) * std::max<size_t>(idx.size(), 1)));
  GB_CUDA_TRY(cudaMalloc(&s->edge_row, sizeof(int) * std::max<size_t>(row.size(), 1)));
  if (!idx.empty()) {
    GB_CUDA_TRY(cudaMemcpy(s->edge_idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice));
    GB_CUDA_TRY(cudaMemcpy(s->edge_row, row.data(), sizeof(int) * row.size(), cudaMemcpyHostToDevice));
  }
  return GB_OK;
}

}  // namespace

extern "C" int gb_adjoint_scatter(gb_system s, const double* x, const double* lambda, double* G,
                                  double* edge_grad) {
  if (!s || !x || !lambda) return GB_BAD_INPUT;
  const int blocks = std::max(1, std::min(device_sm_count() * 8, ceil_div(ceil_div(s->n, 32), 8)));
  if (G) {
    adjoint_scatter_kernel<<<blocks, 256, 0, s->s>>>(s->n, s->ia, s->ja, x, lambda, G);
    GB_CUDA_TRY(cudaGetLastError());
  }
  if (edge_grad) {
    GB_TRY(ensure_edges(s));
    const int g = std::max(1, std::min(device_sm_count() * 8, ceil_div(s->nedges, 256)));
    edge_grad_kernel<<<g, 256, 0, s->s>>>(s->nedges, s->edge_idx, s->edge_row, s->ja, x, lambda,
                                         edge_grad);
    GB_CUDA_TRY(cudaGetLastError());
  }
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  return GB_OK;
}

extern "C" int gb_adjoint_grad(gb_system s, const double* x, const double* g, double* lambda,
                               double* G, double* edge_grad, const gb_pcg_opts* opts,
                               gb_pcg_result* res) {
  if (!s || !x || !g || !lambda) return GB_BAD_INPUT;
  GB_CUDA_TRY(cudaMemsetAsync(lambda, 0, sizeof(double) * s->n, s->s));
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  GB_TRY(gb_pcg_solve(s, g, lambda, opts, nullptr, 0, res));
  return gb_adjoint_scatter(s, x, lambda, G, edge_grad);
}

// CUDA events destroyed on every exit path of the timing helpers below.
namespace {
struct EventSet {
  std::vector<cudaEvent_t> ev;
  int create(int n) {
    ev.assign(n, nullptr);
    for (auto& e : ev) GB_CUDA_TRY(cudaEventCreate(&e));
    return GB_OK;
  }
  cudaEvent_t operator[](int i) const { return ev[i]; }
  ~EventSet() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
};
}  // namespace

// ------------------------------------------------------------ autotuner
namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, int> g_tune_cache;  // (n, nnz, max row) -> rows per bundle
}  // namespace

extern "C" int gb_autotune_spmv(gb_system s, int* best_host) {
  if (!s) return GB_BAD_INPUT;
  int maxrow = 0;
  for (int i = 0; i < s->n; ++i) maxrow = std::max(maxrow, s->h_ia[i + 1] - s->h_ia[i]);
  const auto key = std::make_tuple(s->n, s->nnz, maxrow);
  int best = -1;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto f = g_tune_cache.find(key);
    if (f != g_tune_cache.end()) best = f->second;
  }
  if (best < 0) {
    const int candidates[] = {32, 16, 8, 4};
    float best_ms = 1e30f;
    EventSet ev;
    GB_TRY(ev.create(2));
    const cudaEvent_t e0 = ev[0], e1 = ev[1];
    for (int rpb : candidates) {
      SpmvPlan p;
      GB_TRY(spmv_plan_build(s->n, s->nnz, s->h_ia.data(), &p, rpb));
      struct PlanFree {
        SpmvPlan* p;
        ~PlanFree() { spmv_plan_free(p); }
      } pf{&p};
      for (int w = 0; w < 3; ++w)
        GB_TRY(spmv_axpby<double>(&p, s->n, s->ia, s->ja, s->a, 1.0, s->v64.p0, 0.0, s->v64.q, s->s));
      GB_CUDA_TRY(cudaEventRecord(e0, s->s));
      const int reps = 20;
      for (int r = 0; r < reps; ++r)
        GB_TRY(spmv_axpby<double>(&p, s->n, s->ia, s->ja, s->a, 1.0, s->v64.p0, 0.0, s->v64.q, s->s));
      GB_CUDA_TRY(cudaEventRecord(e1, s->s));
      GB_CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best_ms) {
        best_ms = ms;
        best = rpb;
      }
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = best;
  }
  if (best != s->plan.rows_per_bundle) {
    spmv_plan_free(&s->plan);
    GB_TRY(spmv_plan_build(s->n, s->nnz, s->h_ia.data(), &s->plan, best));
    for (auto& lg : s->loop) {  // captured the old plan
      if (lg.exec) cudaGraphExecDestroy(lg.exec);
      if (lg.graph) cudaGraphDestroy(lg.graph);
      lg = LoopGraph();
    }
    s->loop_key[0] = s->loop_key[1] = -1;
  }
  if (best_host) *best_host = best;
  return GB_OK;
}

// ------------------------------------------------------------ profiling
extern "C" int gb_profile_iteration(gb_system s, const double* b, double* x, int precision,
                                    int iters, char* names_host, int names_len, double* ms_host,
                                    double* bytes_host, int max_kernels, int* count) {
  if (!s || !b || !x || iters <= 0) return GB_BAD_INPUT;
  const size_t bytes = sizeof(double) * s->n;
  GB_TRY(system_ensure_hist(s, iters + 16));
  GB_CUDA_TRY(cudaMemcpyAsync(s->b_int, b, bytes, cudaMemcpyDeviceToDevice, s->s));
  GB_CUDA_TRY(cudaMemcpyAsync(s->v64.x, x, bytes, cudaMemcpyDeviceToDevice, s->s));
  PcgState init;
  memset(&init, 0, sizeof init);
  init.spare0 = 0.0;  // tol 0: never converges during the profile
  init.maxit = iters + 8;
  init.hist_len = s->hist_cap;
  init.flag = 1;
  PcgState* st = s->st;
  if (precision < 0 || precision > 2) return GB_BAD_INPUT;
  if (precision == 0) {
    GB_CUDA_TRY(cudaMemcpyAsync(st, &init, sizeof init, cudaMemcpyHostToDevice, s->s));
    GB_TRY(launch_prologue<double>(s, st, 0, s->b_int));
  } else if (precision == 2) {
    GB_CUDA_TRY(cudaMemcpyAsync(st, &init, sizeof init, cudaMemcpyHostToDevice, s->s));
    GB_TRY(launch_prologue_split(s, st, s->b_int));
  } else {
    PcgState o = init;
    GB_CUDA_TRY(cudaMemcpyAsync(s->st_out, &o, sizeof o, cudaMemcpyHostToDevice, s->s));
    GB_TRY(launch_outer_resid(s, s->b_int, s->v64.x, 1));
    GB_CUDA_TRY(cudaMemcpyAsync(st, &init, sizeof init, cudaMemcpyHostToDevice, s->s));
    GB_TRY(launch_prologue<float>(s, st, 1, s->v32.r));
  }
  GB_CUDA_TRY(cudaStreamSynchronize(s->s));
  ProfHook hook;
  EventSet ev;
  GB_TRY(ev.create(ProfHook::kMax + 1));
  const cudaEvent_t start = ev[0];
  for (int i = 0; i < ProfHook::kMax; ++i) hook.ev[i] = ev[i + 1];
  std::vector<double> acc(ProfHook::kMax, 0.0);
  int nk = 0;
  int rc = GB_OK;
  for (int it = 0; it < iters && rc == GB_OK; ++it) {
    hook.count = 0;
    g_prof = &hook;
    cudaEventRecord(start, s->s);
    rc = precision == 0   ? launch_body<double>(s, st, 0, 0)
         : precision == 2 ? launch_body_split(s, st, 0, 0)
                          : launch_body<float>(s, st, 0, 0);
    g_prof = nullptr;
    if (cudaStreamSynchronize(s->s) != cudaSuccess) rc = GB_CUDA_ERROR;
    nk = hook.count;
    for (int k = 0; k < nk; ++k) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, k == 0 ? start : hook.ev[k - 1], hook.ev[k]);
      acc[k] += ms;
    }
  }
  if (rc != GB_OK) return rc;
  std::string names;
  const int outk = std::min(nk, max_kernels);
  for (int k = 0; k < outk; ++k) {
    if (ms_host) ms_host[k] = acc[k] / iters;
    if (bytes_host) bytes_host[k] = hook.bytes[k];
    if (k) names += ";";
    names += hook.name[k];
  }
  if (names_host && names_len > 0) {
    strncpy(names_host, names.c_str(), names_len - 1);
    names_host[names_len - 1] = 0;
  }
  if (count) *count = outk;
  return GB_OK;
}

