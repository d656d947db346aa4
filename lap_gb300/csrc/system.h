// system.h -- the solver object behind gb_system (device-resident PCG).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "gblap_internal.h"

namespace gb {

struct PcgState;

// Work vectors of one PCG recurrence in precision T.
template <typename T>
struct PcgVectors {
  T *x = nullptr, *r = nullptr, *w = nullptr, *p0 = nullptr, *p1 = nullptr, *q = nullptr;
  T *t = nullptr, *s = nullptr;  // triangular-solve outputs (lower, upper)
};

// One captured solve loop (graph with a device-side while node).
struct LoopGraph {
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
};

enum WKind { WK_NONE = 0, WK_JACOBI = 1, WK_PREC = 2 };

}  // namespace gb

struct gb_system_s {
  int n = 0, nnz = 0;
  const int* ia = nullptr;
  const int* ja = nullptr;
  const double* a = nullptr;
  int prec = GB_PREC_LINE_JACOBI;
  int m = 1, k = 1;
  cudaStream_t s = nullptr;

  std::vector<int> h_ia, h_ja;
  gb::SpmvPlan plan;

  int* dpos = nullptr;   // diagonal position per row
  int* tpos = nullptr;   // transpose position per entry
  double* diag = nullptr;
  double* d_r = nullptr;  // 1/diag (line_jacobi.c / vector_reciprocal)
  float* d_r32 = nullptr;
  float* a32 = nullptr;

  // triangular schedules (GS_std, ichol): L, U for the FP64 solves (exact and
  // FMA form); L32, U32 for the FP32 solves, with tiles twice as tall
  bool tri = false;
  gb::TriPlan L, U;
  gb::TriPlan L32, U32;
  double* fac = nullptr;  // IC(0) factor on A's pattern
  int* fac_done = nullptr;
  int* zero_pivot = nullptr;
  unsigned* fac_ticket = nullptr;
  int zero_pivot_row = 0;

  // strict L / U CSR for the SpMV-only preconditioners (it_jacobi, GS_it, GS_it2)
  int *lia = nullptr, *lja = nullptr, *uia = nullptr, *uja = nullptr;
  double *la = nullptr, *ua = nullptr;
  int lnnz = 0, unnz = 0;
  int *lmap_cpu = nullptr, *umap_cpu = nullptr;  // strict L / U entries -> A entries

  // LAP CPU-layout factor maps (gb_ichol_factor_values) and adjoint maps
  int *lower_idx = nullptr, *lower_row = nullptr;
  int lu_len = 0;
  int *edge_idx = nullptr, *edge_row = nullptr;  // strict-lower entries of A, row-major
  int nedges = 0;
  double* scratch = nullptr;  // small device scalars

  gb::PcgVectors<double> v64;
  gb::PcgVectors<float> v32;
  double* b_int = nullptr;
  double *aux1 = nullptr, *aux2 = nullptr, *aux3 = nullptr;
  double* part = nullptr;
  int part_len = 0;
  int auto_precision = 0;  // the mode gb_pcg_autotune_precision chose (gb_pcg_opts precision -1)
  gb::PcgState* st = nullptr;      // FP64 recurrence (or the inner FP32 one)
  gb::PcgState* st_out = nullptr;  // outer refinement state
  gb::PcgState* st_host = nullptr; // pinned staging
  double* hist = nullptr;
  int hist_cap = 0;
  int* err = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  gb_batch multi = nullptr;       // gb_pcg_solve_multi's shared-matrix batch (a chunk of up to 32)
  gb_batch multi_tail = nullptr;  // ... and the last, shorter chunk when there are more than 32
  int multi_width = 0;            // columns per interleaved chunk (0: 32; gb_pcg_autotune_multi)
  // preconditioner values loaded from caller arrays (gb_system_set_prec_values)
  unsigned long long pat_l = 0, pat_u = 0;  // fingerprints of the L / U layout LAP's pdata holds
  int pl_nnz = 0, pu_nnz = 0;                // their entry counts
  double *pv_l = nullptr, *pv_u = nullptr;   // GS_std: la / ua scattered onto A's pattern
  unsigned long long* hash_dev = nullptr;    // 8 bytes of scratch for pattern_hash
  gb::LoopGraph loop[3];  // [precision]
  int loop_key[3] = {-1, -1, -1};
};

namespace gb {
int system_ensure_hist(gb_system sys, int maxit);
void batch_release(gb_batch bt);
}
