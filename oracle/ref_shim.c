/*
 * ref_shim.c -- links the reference's own NOACC objects (built from the LAP
 * sources by oracle/Makefile into oracle/_ref/libref.so) and exposes one
 * call that replays cg_driver2.c's CPU setup on an in-memory CSR, calls the
 * reference cg(), and hands back x, the iteration count and the residual
 * history.  The reference drivers never write x, so this shim is what makes
 * solution parity against the reference itself possible.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/golden/make_golden.py and the
 * optional reference cross-checks in tests/.
 *
 * Setup replayed: cg_driver2.c:51-61 (split, d), :146-196 (diagonal into L/U
 * for ichol), :354-386 (initialize_ichol, d_r, aux vectors).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "blas.h"
#include "io_utils.h"
#include "simple_blas.h"

static void embed_diag(mmatrix *L, mmatrix *U, const double *D) {
  const int n = L->n;
  int *lja = calloc((size_t)(L->nnz + n) + 1, sizeof(int));
  int *uja = calloc((size_t)(U->nnz + n) + 1, sizeof(int));
  double *la = calloc((size_t)(L->nnz + n) + 1, sizeof(double));
  double *ua = calloc((size_t)(U->nnz + n) + 1, sizeof(double));
  int c = 0;
  for (int i = 0; i < n; ++i) {
    for (int j = L->csr_ia[i]; j < L->csr_ia[i + 1]; ++j) { lja[c] = L->csr_ja[j]; la[c] = L->csr_vals[j]; c++; }
    lja[c] = i; la[c] = D[i]; c++;
  }
  c = 0;
  for (int i = 0; i < n; ++i) {
    uja[c] = i; ua[c] = D[i]; c++;
    for (int j = U->csr_ia[i]; j < U->csr_ia[i + 1]; ++j) { uja[c] = U->csr_ja[j]; ua[c] = U->csr_vals[j]; c++; }
  }
  for (int i = 1; i <= n; ++i) { L->csr_ia[i] += i; U->csr_ia[i] += i; }
  L->nnz += n; U->nnz += n;
  free(L->csr_ja); free(L->csr_vals); free(U->csr_ja); free(U->csr_vals);
  L->csr_ja = lja; L->csr_vals = la; U->csr_ja = uja; U->csr_vals = ua;
}

/* Runs the reference PCG on CSR (ia, ja, a) with rhs b; x holds x0 on entry.
 * If lfac/ufac are non-NULL and prec is "ichol", the reference's L and U
 * factor values are copied out (sizes nnz_strict_lower + n each). */
int ref_solve_csr(int n, int nnz, int *ia, int *ja, double *a, double *b, double *x,
                  const char *prec, double tol, int maxit, int M, int K, int *flag,
                  double *res_hist, double *lfac, double *ufac) {
  mmatrix A, L, U, D;
  memset(&A, 0, sizeof A); memset(&L, 0, sizeof L); memset(&U, 0, sizeof U); memset(&D, 0, sizeof D);
  A.n = A.m = n; A.nnz = n + (nnz - n) / 2; A.nnz_unpacked = nnz;
  A.csr_ia = ia; A.csr_ja = ja; A.csr_vals = a;
  /* split() sizes L/U as A->nnz - A->n, i.e. the count of one strict triangle
   * of a symmetric matrix read from its lower half */
  split(&A, &L, &U, &D);
  double *d = calloc((size_t)n, sizeof(double));
  for (int i = 0; i < n; ++i) d[i] = D.csr_vals[i];
  pdata *p = calloc(1, sizeof(pdata));
  p->n = n; p->prec_op = (char *)prec; p->k = K; p->m = M;
  if (strcmp(prec, "ichol") == 0) {
    embed_diag(&L, &U, d);
    initialize_ichol(n, U.nnz, U.csr_ia, U.csr_ja, U.csr_vals, L.csr_ia, L.csr_ja, L.csr_vals);
    if (lfac) memcpy(lfac, L.csr_vals, sizeof(double) * (size_t)L.nnz);
    if (ufac) memcpy(ufac, U.csr_vals, sizeof(double) * (size_t)U.nnz);
  }
  p->lnnz = L.nnz; p->unnz = U.nnz;
  p->lia = L.csr_ia; p->lja = L.csr_ja; p->la = L.csr_vals;
  p->uia = U.csr_ia; p->uja = U.csr_ja; p->ua = U.csr_vals;
  double *dd = calloc((size_t)n, sizeof(double));
  vector_reciprocal(n, d, dd);
  p->d = d; p->d_r = dd;
  p->aux_vec1 = calloc((size_t)n, sizeof(double));
  p->aux_vec2 = calloc((size_t)n, sizeof(double));
  p->aux_vec3 = calloc((size_t)n, sizeof(double));
  int it = 0;
  *flag = -1;
  cg(n, (real_type)nnz, ia, ja, a, x, b, tol, p, maxit, &it, flag, res_hist);
  fflush(stdout);
  free(d); free(dd); free(p->aux_vec1); free(p->aux_vec2); free(p->aux_vec3); free(p);
  free(L.csr_ia); free(L.csr_ja); free(L.csr_vals);
  free(U.csr_ia); free(U.csr_ja); free(U.csr_vals);
  free(D.csr_ia); free(D.csr_ja); free(D.csr_vals);
  return it;
}

/* Reads a Matrix Market file with the reference reader and converts it with
 * the reference's coo_to_csr; returns malloc'ed arrays (free with ref_free). */
int ref_read_mm_csr(const char *path, int *n, int *nnz, int **ia, int **ja, double **a) {
  mmatrix *A = calloc(1, sizeof(mmatrix));
  read_mm_file(path, A);
  coo_to_csr(A);
  *n = A->n; *nnz = A->nnz_unpacked;
  *ia = A->csr_ia; *ja = A->csr_ja; *a = A->csr_vals;
  free(A);
  return 0;
}

/* Adjacency file -> unweighted/normalised Laplacian with the reference's
 * create_L_and_split (cg_driver.c:26-60). */
int ref_read_laplacian_csr(const char *path, int weighted, int *n, int *nnz, int **ia,
                           int **ja, double **a) {
  mmatrix *A = calloc(1, sizeof(mmatrix)), L, U, D;
  memset(&L, 0, sizeof L); memset(&U, 0, sizeof U); memset(&D, 0, sizeof D);
  read_adjacency_file(path, A);
  coo_to_csr(A);
  create_L_and_split(A, &L, &U, &D, weighted);
  *n = A->n; *nnz = A->nnz_unpacked;
  *ia = A->csr_ia; *ja = A->csr_ja; *a = A->csr_vals;
  free(A);
  return 0;
}

void ref_free(void *p) { free(p); }
