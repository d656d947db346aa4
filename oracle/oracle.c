/*
 * oracle.c -- CPU restatement of kswirydo/LAP's serial PCG path (TEST
 * INFRASTRUCTURE ONLY; see oracle.h).  Built twice by oracle/build.py:
 *   liboracle.so      serial, the parity checker (mirrors simple_blas.c);
 *   liboracle_omp.so  -fopenmp -DORC_OMP: SpMV and dot run multithreaded as
 *                     openmp_blas.c:21-52,171 do; used only to time the
 *                     reference's multicore CPU path.
 * Compile with -ffp-contract=off (no FMA contraction), as the reference's
 * gcc -std=c99 build does, so results are bit-identical to the reference.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef ORC_OMP
#include <omp.h>
#endif

static double wall_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* LAP's OpenMP backend runs its SpMV on a team of exactly 16 threads
 * (openmp_blas.c:37, `omp parallel num_threads(16)`) and its dot product on
 * the default team (openmp_blas.c:171); the mirror does the same. */
#define ORC_SPMV_THREADS 16

int orc_num_threads(void) {
#ifdef ORC_OMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int orc_spmv_threads(void) {
#ifdef ORC_OMP
  return ORC_SPMV_THREADS;
#else
  return 1;
#endif
}

/* ---------------- BLAS-1 (simple_blas.c:4-22, :91-136) ---------------- */

double orc_dot(int n, const double *v, const double *w) {
  double sum = 0.0;
#ifdef ORC_OMP
#pragma omp parallel for reduction(+ : sum) schedule(static)
#endif
  for (int i = 0; i < n; ++i) sum += v[i] * w[i];
  return sum;
}

void orc_scal(int n, double alpha, double *v) {
  for (int i = 0; i < n; ++i) v[i] *= alpha;
}

void orc_axpy(int n, double alpha, const double *x, double *y) {
  for (int i = 0; i < n; ++i) y[i] += alpha * x[i];
}

void orc_vec_vec(int n, const double *x, const double *y, double *res) {
  for (int i = 0; i < n; ++i) res[i] = x[i] * y[i];
}

void orc_vector_reciprocal(int n, const double *v, double *res) {
  for (int i = 0; i < n; ++i) res[i] = (v[i] != 0.0) ? 1.0 / v[i] : 0.0;
}

void orc_vector_sqrt(int n, const double *v, double *res) {
  for (int i = 0; i < n; ++i) res[i] = (v[i] >= 0.0) ? sqrt(v[i]) : 0.0;
}

void orc_vec_copy(int n, const double *src, double *dest) {
  for (int i = 0; i < n; ++i) dest[i] = src[i];
}

void orc_vec_zero(int n, double *v) {
  for (int i = 0; i < n; ++i) v[i] = 0.0;
}

/* ---------------- sparse kernels (simple_blas.c:24-85) ---------------- */

/* y = beta*y, then y += (alpha*a_j)*x_col in row order. */
void orc_csr_matvec(int n, int nnz, const int *ia, const int *ja, const double *a,
                    const double *x, double *y, const double *alpha_p,
                    const double *beta_p) {
  (void)nnz;
  const double alpha = *alpha_p, beta = *beta_p;
#ifdef ORC_OMP
#pragma omp parallel for num_threads(ORC_SPMV_THREADS) schedule(static)
#endif
  for (int i = 0; i < n; ++i) {
    double acc = y[i] * beta;
    for (int j = ia[i]; j < ia[i + 1]; ++j) acc += alpha * a[j] * x[ja[j]];
    y[i] = acc;
  }
}

/* Forward substitution with a separate diagonal: strict-lower CSR. */
void orc_lower_solve(int n, int nnz, const int *lia, const int *lja, const double *la,
                     const double *diag, const double *x, double *result) {
  (void)nnz;
  for (int i = 0; i < n; ++i) {
    double acc = x[i];
    for (int j = lia[i]; j < lia[i + 1]; ++j) acc -= la[j] * result[lja[j]];
    result[i] = acc / diag[i];
  }
}

/* Backward substitution with a separate diagonal: strict-upper CSR. */
void orc_upper_solve(int n, int nnz, const int *uia, const int *uja, const double *ua,
                     const double *diag, const double *x, double *result) {
  (void)nnz;
  for (int i = n - 1; i >= 0; --i) {
    double acc = x[i];
    for (int j = uia[i]; j < uia[i + 1]; ++j) acc -= ua[j] * result[uja[j]];
    result[i] = acc / diag[i];
  }
}

/* ---------------- IC(0) (simple_blas.c:139-223) ---------------- */

void orc_ichol_factor(int n, int nnzU, const int *uia, const int *uja, double *ua,
                      const int *lia, const int *lja, double *la) {
  (void)lja;
  /* right-looking sweep over the upper factor, row i eliminates into rows j > i */
  for (int i = 0; i < n; ++i) {
    const int d = uia[i];
    ua[d] = sqrt(ua[d]);
    for (int m = d + 1; m < uia[i + 1]; ++m) ua[m] = ua[m] / ua[d];
    for (int m = d + 1; m < uia[i + 1]; ++m) {
      const int j = uja[m];
      for (int k = uia[j]; k < uia[j + 1]; ++k) {
        for (int l = m; l < uia[i + 1]; ++l) {
          if (uja[l] == uja[k]) ua[k] -= ua[m] * ua[l];
        }
      }
    }
  }
  /* transpose U into L: entries of column c of U land in row c of L in
   * increasing source-row order */
  int *fill = (int *)calloc((size_t)(nnzU > n ? nnzU : n) + 1, sizeof(int));
  for (int i = 0; i < n; ++i) {
    for (int j = uia[i]; j < uia[i + 1]; ++j) {
      const int row = uja[j];
      la[lia[row] + fill[row]] = ua[j];
      fill[row]++;
    }
  }
  free(fill);
}

void orc_ichol_apply(orc_pdata *p, const double *x, double *y) {
  const int n = p->n;
  double *t = p->aux_vec1;
  for (int i = 0; i < n; ++i) {
    double acc = x[i];
    for (int j = p->lia[i]; j < p->lia[i + 1]; ++j) {
      const int col = p->lja[j];
      if (col != i) acc -= p->la[j] * t[col];
    }
    t[i] = acc / p->la[p->lia[i + 1] - 1];
  }
  for (int i = n - 1; i >= 0; --i) {
    double acc = t[i];
    for (int j = p->uia[i]; j < p->uia[i + 1]; ++j) {
      const int col = p->uja[j];
      if (col != i) acc -= p->ua[j] * y[col];
    }
    y[i] = acc / p->ua[p->uia[i]];
  }
}

/* ---------------- preconditioners (GS.c, it_jacobi.c, line_jacobi.c) ---------------- */

void orc_line_jacobi(orc_pdata *p, const double *in, double *out) {
  orc_vec_vec(p->n, p->d_r, in, out);
}

void orc_it_jacobi(orc_pdata *p, const double *in, double *out) {
  const int n = p->n;
  const double one = 1.0, zero = 0.0;
  orc_vec_zero(n, out);
  for (int s = 0; s < p->k; ++s) {
    orc_csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, out, p->aux_vec1, &one, &zero);
    orc_csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, out, p->aux_vec2, &one, &zero);
    /* it_jacobi.c:339 passes the float literal 1.0f; it widens to exactly 1.0 */
    orc_axpy(n, 1.0, p->aux_vec1, p->aux_vec2);
    orc_vec_copy(n, in, out);
    orc_axpy(n, -1.0, p->aux_vec2, out);
    orc_vec_vec(n, out, p->d_r, out);
  }
}

void orc_GS_std(const int *ia, const int *ja, const double *a, int nnzA, orc_pdata *p,
                const double *in, double *out) {
  const int n = p->n;
  const double one = 1.0, minusone = -1.0;
  orc_vec_zero(n, out);
  for (int s = 0; s < p->k; ++s) {
    orc_vec_copy(n, in, p->aux_vec2);
    orc_csr_matvec(n, nnzA, ia, ja, a, out, p->aux_vec2, &minusone, &one);
    orc_lower_solve(n, p->lnnz, p->lia, p->lja, p->la, p->d, p->aux_vec2, p->aux_vec1);
    orc_axpy(n, 1.0, p->aux_vec1, out);
  }
  for (int s = 0; s < p->k; ++s) {
    orc_vec_copy(n, in, p->aux_vec2);
    orc_csr_matvec(n, nnzA, ia, ja, a, out, p->aux_vec2, &minusone, &one);
    orc_upper_solve(n, p->unnz, p->uia, p->uja, p->ua, p->d, p->aux_vec2, p->aux_vec1);
    orc_axpy(n, 1.0, p->aux_vec1, out);
  }
}

void orc_GS_it(const int *ia, const int *ja, const double *a, int nnzA, orc_pdata *p,
               const double *in, double *out) {
  const int n = p->n;
  const double one = 1.0, minusone = -1.0;
  orc_vec_zero(n, out);
  for (int o = 0; o < p->m; ++o) {
    orc_vec_copy(n, in, p->aux_vec2);
    orc_csr_matvec(n, nnzA, ia, ja, a, out, p->aux_vec2, &minusone, &one);
    orc_vec_vec(n, p->aux_vec2, p->d_r, p->aux_vec1);
    for (int s = 0; s < p->k; ++s) {
      orc_vec_copy(n, p->aux_vec2, p->aux_vec3);
      orc_csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, p->aux_vec1, p->aux_vec3, &minusone,
                     &one);
      orc_vec_vec(n, p->aux_vec3, p->d_r, p->aux_vec1);
    }
    for (int s = 0; s < p->k; ++s) {
      orc_vec_copy(n, p->aux_vec2, p->aux_vec3);
      orc_csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, p->aux_vec1, p->aux_vec3, &minusone,
                     &one);
      orc_vec_vec(n, p->aux_vec3, p->d_r, p->aux_vec1);
    }
    orc_axpy(n, 1.0, p->aux_vec1, out);
  }
}

void orc_GS_it2(const int *ia, const int *ja, const double *a, int nnzA, orc_pdata *p,
                const double *in, double *out) {
  (void)ia; (void)ja; (void)a; (void)nnzA;
  const int n = p->n;
  const double one = 1.0, zero = 0.0, minusone = -1.0;
  double *v1 = p->aux_vec1, *v2 = p->aux_vec2, *v3 = p->aux_vec3;
  orc_vec_vec(n, in, p->d_r, v1);
  for (int o = 0; o < p->m; ++o) {
    /* one Jacobi-style step on (L+U) */
    orc_csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, v1, v2, &one, &zero);
    orc_csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, v1, v3, &one, &zero);
    orc_axpy(n, 1.0, v3, v2);
    orc_vec_copy(n, in, v3);
    orc_axpy(n, -1.0, v2, v3);
    orc_vec_vec(n, v3, p->d_r, v2);
    /* r = b - L y; then k steps y = D^-1 (r - U y) */
    orc_vec_copy(n, in, v3);
    orc_csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, v2, v3, &minusone, &one);
    for (int s = 0; s < p->k; ++s) {
      orc_vec_copy(n, v3, v1);
      orc_csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, v2, v1, &minusone, &one);
      orc_vec_vec(n, p->d_r, v1, v2);
    }
    /* r = b - U y; then k steps y = D^-1 (r - L y) */
    orc_vec_copy(n, in, v3);
    orc_csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, v2, v3, &minusone, &one);
    for (int s = 0; s < p->k; ++s) {
      orc_vec_copy(n, v3, v1);
      orc_csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, v2, v1, &minusone, &one);
      orc_vec_vec(n, p->d_r, v1, v2);
    }
    orc_vec_copy(n, v2, v1);
  }
  orc_vec_copy(n, v2, out);
}

void orc_prec_function(const int *ia, const int *ja, const double *a, int nnzA, orc_pdata *p,
                       const double *x, double *y) {
  /* the reference tests every name in turn and leaves y untouched for an
   * unknown one (prec.c:6-45) */
  if (strcmp(p->prec_op, "it_jacobi") == 0) orc_it_jacobi(p, x, y);
  if (strcmp(p->prec_op, "line_jacobi") == 0) orc_line_jacobi(p, x, y);
  if (strcmp(p->prec_op, "GS_std") == 0) orc_GS_std(ia, ja, a, nnzA, p, x, y);
  if (strcmp(p->prec_op, "GS_it") == 0) orc_GS_it(ia, ja, a, nnzA, p, x, y);
  if (strcmp(p->prec_op, "ichol") == 0) orc_ichol_apply(p, x, y);
  if (strcmp(p->prec_op, "GS_it2") == 0) orc_GS_it2(ia, ja, a, nnzA, p, x, y);
  if (strcmp(p->prec_op, "none") == 0) orc_vec_copy(p->n, x, y);
}

/* ---------------- PCG (cg.c:5-140) ---------------- */

int orc_cg(int n, int nnz, const int *ia, const int *ja, const double *a, double *x,
           const double *b, double tol, orc_pdata *p, int maxit, int *flag,
           double *res_hist, double *true_res, int max_iters_run) {
  double *r = (double *)calloc((size_t)n, sizeof(double));
  double *w = (double *)calloc((size_t)n, sizeof(double));
  double *pv = (double *)calloc((size_t)n, sizeof(double));
  double *q = (double *)calloc((size_t)n, sizeof(double));
  const double one = 1.0, zero = 0.0;
  double rho = 0.0, rho_prev = 0.0;
  int iter = 0, done = 0;

  orc_csr_matvec(n, nnz, ia, ja, a, x, r, &one, &zero);
  orc_axpy(n, -1.0, b, r);
  orc_scal(n, -1.0, r);
  res_hist[0] = sqrt(orc_dot(n, r, r));
  const double tolrel = tol * res_hist[0];
  *flag = 1;

  while (!done) {
    orc_prec_function(ia, ja, a, nnz, p, r, w);
    rho = orc_dot(n, r, w);
    if (iter == 0) {
      orc_vec_copy(n, w, pv);
    } else {
      const double beta = rho / rho_prev;
      orc_scal(n, beta, pv);
      orc_axpy(n, 1.0, w, pv);
    }
    orc_csr_matvec(n, nnz, ia, ja, a, pv, q, &one, &zero);
    const double alpha = rho / orc_dot(n, pv, q);
    orc_axpy(n, alpha, pv, x);
    orc_axpy(n, -1.0 * alpha, q, r);
    iter++;
    res_hist[iter] = sqrt(orc_dot(n, r, r));
    if (res_hist[iter] < tolrel) {
      *flag = 0;
      done = 1;
      if (true_res) {
        orc_csr_matvec(n, nnz, ia, ja, a, x, r, &one, &zero);
        orc_axpy(n, -1.0, b, r);
        *true_res = sqrt(orc_dot(n, r, r));
      }
    } else if (iter > maxit) {
      *flag = 1;
      done = 1;
    } else if (max_iters_run > 0 && iter >= max_iters_run) {
      *flag = 1;
      done = 1;
    }
    rho_prev = rho;
  }
  free(r); free(w); free(pv); free(q);
  return iter;
}

/* ---------------- Matrix Market I/O (io_utils.c) ---------------- */

static int read_header(FILE *f, char *line, size_t len, int *pattern, int *sym) {
  if (!fgets(line, (int)len, f)) return -1;
  if (pattern) *pattern = strstr(line, "pattern") != NULL;
  if (sym) *sym = strstr(line, "symmetric") != NULL;
  while (line[0] == '%') {
    if (!fgets(line, (int)len, f)) return -1;
  }
  return 0;
}

int orc_read_mm(const char *path, orc_mmatrix *A) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  char line[256];
  int pattern = 0, sym = 0;
  memset(A, 0, sizeof(*A));
  if (read_header(f, line, sizeof line, &pattern, &sym)) { fclose(f); return -1; }
  A->symmetric = sym;
  long n = 0, m = 0, nnz = 0;
  sscanf(line, "%ld %ld %ld", &n, &m, &nnz);
  A->n = (int)n; A->m = (int)m; A->nnz = (int)nnz;
  A->coo_vals = (double *)calloc((size_t)nnz + 1, sizeof(double));
  A->coo_rows = (int *)calloc((size_t)nnz + 1, sizeof(int));
  A->coo_cols = (int *)calloc((size_t)nnz + 1, sizeof(int));
  int i = 0;
  while (i < nnz && fgets(line, sizeof line, f)) {
    int r = 0, c = 0; double v = 1.0;
    if (!pattern) sscanf(line, "%d %d %lf", &r, &c, &v);
    else sscanf(line, "%d %d", &r, &c);
    A->coo_vals[i] = v; A->coo_rows[i] = r - 1; A->coo_cols[i] = c - 1;
    i++;
  }
  fclose(f);
  return 0;
}

int orc_read_adjacency(const char *path, orc_mmatrix *A) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  char line[256];
  int pattern = 0;
  memset(A, 0, sizeof(*A));
  if (read_header(f, line, sizeof line, &pattern, NULL)) { fclose(f); return -1; }
  A->symmetric = 1;
  long n = 0, m = 0, nnz = 0;
  sscanf(line, "%ld %ld %ld", &n, &m, &nnz);
  A->n = (int)n; A->m = (int)m; A->nnz = (int)nnz;
  A->coo_vals = (double *)calloc((size_t)(nnz + n) + 1, sizeof(double));
  A->coo_rows = (int *)calloc((size_t)(nnz + n) + 1, sizeof(int));
  A->coo_cols = (int *)calloc((size_t)(nnz + n) + 1, sizeof(int));
  int i = 0;
  while (i < nnz && fgets(line, sizeof line, f)) {
    int r = 0, c = 0; double v = 1.0;
    if (!pattern) sscanf(line, "%d %d %lf", &r, &c, &v);
    else sscanf(line, "%d %d", &r, &c);
    A->coo_vals[i] = v; A->coo_rows[i] = r - 1; A->coo_cols[i] = c - 1;
    i++;
  }
  /* unit diagonal placeholders, overwritten by the Laplacian builder */
  for (int j = 0; j < A->n; ++j) {
    A->coo_rows[i] = j; A->coo_cols[i] = j; A->coo_vals[i] = 1.0; i++;
  }
  A->nnz += A->n;
  fclose(f);
  return 0;
}

typedef struct { double value; int idx; } orc_iv;
static int iv_cmp(const void *pa, const void *pb) {
  const orc_iv *a = (const orc_iv *)pa, *b = (const orc_iv *)pb;
  return a->idx < b->idx ? -1 : a->idx > b->idx;
}

void orc_coo_to_csr(orc_mmatrix *A) {
  const int n = A->n;
  int *cnt = (int *)calloc((size_t)n + 1, sizeof(int));
  int total = 0;
  for (int i = 0; i < A->nnz; ++i) {
    cnt[A->coo_rows[i]]++; total++;
    if (A->symmetric && A->coo_rows[i] != A->coo_cols[i]) { cnt[A->coo_cols[i]]++; total++; }
  }
  A->nnz_unpacked = total;
  A->csr_ia = (int *)calloc((size_t)n + 1, sizeof(int));
  A->csr_ja = (int *)calloc((size_t)total + 1, sizeof(int));
  A->csr_vals = (double *)calloc((size_t)total + 1, sizeof(double));
  orc_iv *tmp = (orc_iv *)calloc((size_t)total + 1, sizeof(orc_iv));
  for (int i = 1; i <= n; ++i) A->csr_ia[i] = A->csr_ia[i - 1] + cnt[i - 1];
  int *fill = (int *)calloc((size_t)n + 1, sizeof(int));
  for (int i = 0; i < A->nnz; ++i) {
    int r = A->coo_rows[i];
    tmp[A->csr_ia[r] + fill[r]].idx = A->coo_cols[i];
    tmp[A->csr_ia[r] + fill[r]].value = A->coo_vals[i];
    fill[r]++;
    if (A->symmetric && A->coo_rows[i] != A->coo_cols[i]) {
      r = A->coo_cols[i];
      tmp[A->csr_ia[r] + fill[r]].idx = A->coo_rows[i];
      tmp[A->csr_ia[r] + fill[r]].value = A->coo_vals[i];
      fill[r]++;
    }
  }
  /* qsort per row; equal columns (duplicates) are not merged, as in the
   * reference, and their relative order is whatever qsort leaves */
  for (int i = 0; i < n; ++i)
    qsort(tmp + A->csr_ia[i], (size_t)(A->csr_ia[i + 1] - A->csr_ia[i]), sizeof(orc_iv), iv_cmp);
  for (int i = 0; i < total; ++i) { A->csr_ja[i] = tmp[i].idx; A->csr_vals[i] = tmp[i].value; }
  free(cnt); free(fill); free(tmp);
  free(A->coo_rows); free(A->coo_cols); free(A->coo_vals);
  A->coo_rows = NULL; A->coo_cols = NULL; A->coo_vals = NULL;
}

int orc_read_rhs(const char *path, double *rhs, int n) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  char line[256];
  if (read_header(f, line, sizeof line, NULL, NULL)) { fclose(f); return -1; }
  long N = 0, m = 0;
  sscanf(line, "%ld %ld", &N, &m);
  int i = 0;
  while (i != N && i < n && fgets(line, sizeof line, f)) {
    double v = 0.0;
    sscanf(line, "%lf", &v);
    rhs[i++] = v;
  }
  fclose(f);
  return i;
}

static void alloc_split(orc_mmatrix *M, int n, int cap) {
  memset(M, 0, sizeof(*M));
  M->n = n; M->m = n;
  M->csr_ia = (int *)calloc((size_t)n + 1, sizeof(int));
  M->csr_ja = (int *)calloc((size_t)cap + 1, sizeof(int));
  M->csr_vals = (double *)calloc((size_t)cap + 1, sizeof(double));
}

void orc_split(const orc_mmatrix *A, orc_mmatrix *L, orc_mmatrix *U, double *D) {
  const int n = A->n;
  const int cap = A->nnz_unpacked;
  alloc_split(L, n, cap);
  alloc_split(U, n, cap);
  int il = 0, iu = 0;
  for (int i = 0; i < n; ++i) {
    L->csr_ia[i] = il; U->csr_ia[i] = iu;
    for (int j = A->csr_ia[i]; j < A->csr_ia[i + 1]; ++j) {
      const int col = A->csr_ja[j];
      if (col == i) D[i] = A->csr_vals[j];
      if (i < col) { U->csr_ja[iu] = col; U->csr_vals[iu] = A->csr_vals[j]; iu++; }
      if (i > col) { L->csr_ja[il] = col; L->csr_vals[il] = A->csr_vals[j]; il++; }
    }
  }
  L->csr_ia[n] = il; U->csr_ia[n] = iu;
  L->nnz = L->nnz_unpacked = il;
  U->nnz = U->nnz_unpacked = iu;
}

void orc_create_L_and_split(orc_mmatrix *A, orc_mmatrix *L, orc_mmatrix *U, double *D,
                            int weighted) {
  const int n = A->n;
  int *deg = (int *)calloc((size_t)n + 1, sizeof(int));
  for (int i = 0; i < n; ++i) {
    deg[i] = -1; /* the stored unit diagonal does not count */
    for (int j = A->csr_ia[i]; j < A->csr_ia[i + 1]; ++j) deg[i] += A->csr_vals[j];
  }
  for (int i = 0; i < n; ++i) {
    const double dsq = weighted ? 1.0 / sqrt((double)deg[i]) : 0.0;
    for (int j = A->csr_ia[i]; j < A->csr_ia[i + 1]; ++j) {
      const int col = A->csr_ja[j];
      if (col == i) {
        A->csr_vals[j] = weighted ? 1.0 : (double)deg[i];
      } else if (!weighted) {
        A->csr_vals[j] = (-1.0) * A->csr_vals[j];
      } else {
        A->csr_vals[j] = (-1.0) * A->csr_vals[j] * dsq * (1.0 / sqrt((double)deg[col]));
      }
    }
  }
  free(deg);
  orc_split(A, L, U, D);
}

void orc_embed_diagonal(orc_mmatrix *L, orc_mmatrix *U, const double *D) {
  const int n = L->n;
  int *lja = (int *)calloc((size_t)(L->nnz + n) + 1, sizeof(int));
  int *uja = (int *)calloc((size_t)(U->nnz + n) + 1, sizeof(int));
  double *la = (double *)calloc((size_t)(L->nnz + n) + 1, sizeof(double));
  double *ua = (double *)calloc((size_t)(U->nnz + n) + 1, sizeof(double));
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
  L->nnz_unpacked = L->nnz; U->nnz_unpacked = U->nnz;
  free(L->csr_ja); free(L->csr_vals); free(U->csr_ja); free(U->csr_vals);
  L->csr_ja = lja; L->csr_vals = la; U->csr_ja = uja; U->csr_vals = ua;
}

void orc_free_matrix(orc_mmatrix *A) {
  free(A->coo_rows); free(A->coo_cols); free(A->coo_vals);
  free(A->csr_ia); free(A->csr_ja); free(A->csr_vals);
  memset(A, 0, sizeof(*A));
}

void orc_free(void *p) { free(p); }

/* ---------------- one-call solve (cg_driver2.c NOACC path) ---------------- */

/* One preconditioner application y = M^{-1} x after cg_driver2.c's NOACC
 * setup (mode 0 = full run through orc_cg, used by orc_solve_csr; mode 1 =
 * apply only). */
static int run_csr(int n, int nnz, const int *ia, const int *ja, const double *a,
                   const double *b, double *x, const char *prec, double tol, int maxit,
                   int M, int K, int *flag, double *res_hist, double *true_res,
                   int max_iters_run, double *setup_s, double *solve_s, int apply_only,
                   const double *px, double *py);

int orc_prec_apply_csr(int n, int nnz, const int *ia, const int *ja, const double *a,
                       const char *prec, int M, int K, const double *x, double *y) {
  return run_csr(n, nnz, ia, ja, a, NULL, NULL, prec, 0.0, 0, M, K, NULL, NULL, NULL, 0, NULL,
                 NULL, 1, x, y);
}

int orc_solve_csr(int n, int nnz, const int *ia, const int *ja, const double *a,
                  const double *b, double *x, const char *prec, double tol, int maxit,
                  int M, int K, int *flag, double *res_hist, double *true_res,
                  int max_iters_run, double *setup_s, double *solve_s) {
  return run_csr(n, nnz, ia, ja, a, b, x, prec, tol, maxit, M, K, flag, res_hist, true_res,
                 max_iters_run, setup_s, solve_s, 0, NULL, NULL);
}

static int run_csr(int n, int nnz, const int *ia, const int *ja, const double *a,
                  const double *b, double *x, const char *prec, double tol, int maxit,
                  int M, int K, int *flag, double *res_hist, double *true_res,
                   int max_iters_run, double *setup_s, double *solve_s, int apply_only,
                   const double *px, double *py) {
  const double t0 = wall_s();
  orc_mmatrix A, L, U;
  memset(&A, 0, sizeof A);
  A.n = A.m = n; A.nnz = A.nnz_unpacked = nnz;
  A.csr_ia = (int *)ia; A.csr_ja = (int *)ja; A.csr_vals = (double *)a;
  double *d = (double *)calloc((size_t)n + 1, sizeof(double));
  orc_split(&A, &L, &U, d);
  if (strcmp(prec, "ichol") == 0) {
    orc_embed_diagonal(&L, &U, d);
    orc_ichol_factor(n, U.nnz, U.csr_ia, U.csr_ja, U.csr_vals, L.csr_ia, L.csr_ja, L.csr_vals);
  }
  orc_pdata p;
  memset(&p, 0, sizeof p);
  p.n = n; p.prec_op = prec; p.m = M; p.k = K;
  p.lia = L.csr_ia; p.lja = L.csr_ja; p.la = L.csr_vals; p.lnnz = L.nnz;
  p.uia = U.csr_ia; p.uja = U.csr_ja; p.ua = U.csr_vals; p.unnz = U.nnz;
  p.d = d;
  p.d_r = (double *)calloc((size_t)n + 1, sizeof(double));
  orc_vector_reciprocal(n, d, p.d_r);
  p.aux_vec1 = (double *)calloc((size_t)n + 1, sizeof(double));
  p.aux_vec2 = (double *)calloc((size_t)n + 1, sizeof(double));
  p.aux_vec3 = (double *)calloc((size_t)n + 1, sizeof(double));
  const double t1 = wall_s();
  const int it = apply_only ? (orc_prec_function(ia, ja, a, nnz, &p, px, py), 0)
                            : orc_cg(n, nnz, ia, ja, a, x, b, tol, &p, maxit, flag, res_hist,
                                     true_res, max_iters_run);
  const double t2 = wall_s();
  if (setup_s) *setup_s = t1 - t0;
  if (solve_s) *solve_s = t2 - t1;
  free(d); free(p.d_r); free(p.aux_vec1); free(p.aux_vec2); free(p.aux_vec3);
  free(L.csr_ia); free(L.csr_ja); free(L.csr_vals);
  free(U.csr_ia); free(U.csr_ja); free(U.csr_vals);
  return it;
}
