// pcg.h -- launchers of the fused PCG kernels (pcg.cu) and the composed
// preconditioners (precond.cu).
#pragma once

#include "gblap_internal.h"
#include "system.h"

namespace gb {

int prec_wkind(int prec, int k);
bool prec_fused_tri(int prec, int k);
int part_len_needed(gb_system sys);

template <typename T>
int launch_prologue(gb_system sys, PcgState* st, int x_zero, const T* b);
template <typename T>
int launch_body(gb_system sys, PcgState* st, cudaGraphConditionalHandle cond, int has_cond);

// Split precision (ichol, GS_std with k = 1): FP64 recurrence, FP32 SpMV
// values and FP32 triangular solves.  The resume replaces nothing itself:
// launch_outer_resid64 writes the FP64 true residual into the recurrence's
// r first.
int launch_prologue_split(gb_system sys, PcgState* st, const double* b);
int launch_body_split(gb_system sys, PcgState* st, cudaGraphConditionalHandle cond, int has_cond);
int launch_resume_split(gb_system sys, PcgState* st, double delta);
int launch_outer_resid64(gb_system sys, const double* b, const double* x, int first);

int launch_true_resid(gb_system sys, const double* b, const double* x, double* out2);
int launch_outer_resid(gb_system sys, const double* b, const double* x, int first);
int launch_add_correction(gb_system sys, double* x);
// Resumes a paused recurrence after its residual was replaced (mixed
// precision): clears the pause, sets the next pause threshold to
// delta*||r_true|| and recomputes w = M^-1 r and rho for the new r.
template <typename T>
int launch_resume(gb_system sys, PcgState* st, double delta);

// LAP's preconditioners that are compositions of SpMV / BLAS-1 calls
// (it_jacobi.c, GS.c GS_it / GS_it2, GS_std with k > 1, and line_jacobi /
// none for completeness): y = M^{-1} x, FP64, on the system stream.
int apply_prec_composed(gb_system sys, const double* x, double* y);
// Any preconditioner (including the sync-free GS_std / ichol solves).
int apply_prec(gb_system sys, const double* x, double* y);

// Per-kernel timing hook used by gb_profile_iteration: while set, every PCG
// kernel launch is followed by an event record on the system stream.
struct ProfHook {
  static constexpr int kMax = 32;
  int count = 0;
  cudaEvent_t ev[kMax];
  const char* name[kMax];
  double bytes[kMax];
};
extern ProfHook* g_prof;
void prof_mark(cudaStream_t s, const char* name, double bytes);

}  // namespace gb
