// precond.cu -- LAP's preconditioners as compositions of the library's
// kernels, in the reference's call order (so each elementwise result equals
// the reference's): line_jacobi.c:3-7, it_jacobi.c:4-33, GS.c:5-159,
// simple_blas.c:184-223 (IC(0) apply), prec.c:6-45 (dispatch).
#include "gb_common.cuh"
#include "kernels.h"
#include "pcg.h"
#include "sptrsv.h"
#include "system.h"

namespace gb {

static int spmv_L(gb_system s, const double* x, double* y, double alpha, double beta) {
  return spmv_axpby<double>(nullptr, s->n, s->lia, s->lja, s->la, alpha, x, beta, y, s->s);
}
static int spmv_U(gb_system s, const double* x, double* y, double alpha, double beta) {
  return spmv_axpby<double>(nullptr, s->n, s->uia, s->uja, s->ua, alpha, x, beta, y, s->s);
}
static int spmv_A(gb_system s, const double* x, double* y, double alpha, double beta) {
  return spmv_axpby<double>(&s->plan, s->n, s->ia, s->ja, s->a, alpha, x, beta, y, s->s);
}

int apply_prec_composed(gb_system sys, const double* in, double* out) {
  const int n = sys->n;
  cudaStream_t st = sys->s;
  double *v1 = sys->aux1, *v2 = sys->aux2, *v3 = sys->aux3;
  switch (sys->prec) {
    case GB_PREC_NONE:
      return copy_dev(n, in, out, st);
    case GB_PREC_LINE_JACOBI:
      return vec_vec_dev(n, sys->d_r, in, out, st);
    case GB_PREC_IT_JACOBI: {
      // it_jacobi.c:13-31
      GB_TRY(fill_dev(n, 0.0, out, st));
      for (int i = 0; i < sys->k; ++i) {
        GB_TRY(spmv_L(sys, out, v1, 1.0, 0.0));
        GB_TRY(spmv_U(sys, out, v2, 1.0, 0.0));
        GB_TRY(axpy_dev(n, 1.0, v1, v2, st));
        GB_TRY(copy_dev(n, in, out, st));
        GB_TRY(axpy_dev(n, -1.0, v2, out, st));
        GB_TRY(vec_vec_dev(n, out, sys->d_r, out, st));
      }
      return GB_OK;
    }
    case GB_PREC_GS_IT: {
      // GS.c:55-91
      GB_TRY(fill_dev(n, 0.0, out, st));
      for (int j = 0; j < sys->m; ++j) {
        GB_TRY(copy_dev(n, in, v2, st));
        GB_TRY(spmv_A(sys, out, v2, -1.0, 1.0));
        GB_TRY(vec_vec_dev(n, v2, sys->d_r, v1, st));
        for (int i = 0; i < sys->k; ++i) {
          GB_TRY(copy_dev(n, v2, v3, st));
          GB_TRY(spmv_L(sys, v1, v3, -1.0, 1.0));
          GB_TRY(vec_vec_dev(n, v3, sys->d_r, v1, st));
        }
        for (int i = 0; i < sys->k; ++i) {
          GB_TRY(copy_dev(n, v2, v3, st));
          GB_TRY(spmv_U(sys, v1, v3, -1.0, 1.0));
          GB_TRY(vec_vec_dev(n, v3, sys->d_r, v1, st));
        }
        GB_TRY(axpy_dev(n, 1.0, v1, out, st));
      }
      return GB_OK;
    }
    case GB_PREC_GS_IT2: {
      // GS.c:105-158
      GB_TRY(vec_vec_dev(n, in, sys->d_r, v1, st));
      for (int j = 0; j < sys->m; ++j) {
        GB_TRY(spmv_L(sys, v1, v2, 1.0, 0.0));
        GB_TRY(spmv_U(sys, v1, v3, 1.0, 0.0));
        GB_TRY(axpy_dev(n, 1.0, v3, v2, st));
        GB_TRY(copy_dev(n, in, v3, st));
        GB_TRY(axpy_dev(n, -1.0, v2, v3, st));
        GB_TRY(vec_vec_dev(n, v3, sys->d_r, v2, st));
        GB_TRY(copy_dev(n, in, v3, st));
        GB_TRY(spmv_L(sys, v2, v3, -1.0, 1.0));
        for (int i = 0; i < sys->k; ++i) {
          GB_TRY(copy_dev(n, v3, v1, st));
          GB_TRY(spmv_U(sys, v2, v1, -1.0, 1.0));
          GB_TRY(vec_vec_dev(n, sys->d_r, v1, v2, st));
        }
        GB_TRY(copy_dev(n, in, v3, st));
        GB_TRY(spmv_U(sys, v2, v3, -1.0, 1.0));
        for (int i = 0; i < sys->k; ++i) {
          GB_TRY(copy_dev(n, v3, v1, st));
          GB_TRY(spmv_L(sys, v2, v1, -1.0, 1.0));
          GB_TRY(vec_vec_dev(n, sys->d_r, v1, v2, st));
        }
        GB_TRY(copy_dev(n, v2, v1, st));
      }
      return copy_dev(n, v2, out, st);
    }
    case GB_PREC_GS_STD: {
      // GS.c:11-41: k forward sweeps with (D+L), then k backward with (D+U)
      GB_TRY(fill_dev(n, 0.0, out, st));
      for (int i = 0; i < sys->k; ++i) {
        GB_TRY(copy_dev(n, in, v2, st));
        GB_TRY(spmv_A(sys, out, v2, -1.0, 1.0));
        GB_TRY(tri_solve_plain(&sys->L, v2, v1, sys->err, st));
        GB_TRY(axpy_dev(n, 1.0, v1, out, st));
      }
      for (int i = 0; i < sys->k; ++i) {
        GB_TRY(copy_dev(n, in, v2, st));
        GB_TRY(spmv_A(sys, out, v2, -1.0, 1.0));
        GB_TRY(tri_solve_plain(&sys->U, v2, v1, sys->err, st));
        GB_TRY(axpy_dev(n, 1.0, v1, out, st));
      }
      return GB_OK;
    }
    case GB_PREC_ICHOL:
      // simple_blas.c:200-221: L^{-1} then (L^T)^{-1}
      GB_TRY(tri_solve_plain(&sys->L, in, v1, sys->err, st));
      return tri_solve_plain(&sys->U, v1, out, sys->err, st);
  }
  return GB_BAD_INPUT;
}

int apply_prec(gb_system sys, const double* x, double* y) { return apply_prec_composed(sys, x, y); }

}  // namespace gb
