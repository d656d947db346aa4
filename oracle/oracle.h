/*
 * oracle.h -- CPU restatement of kswirydo/LAP's serial (NOACC) PCG path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: the pytest suite, the
 * smoke entry point and bench.py's CPU-baseline leg call it.  The product
 * (lap_gb300/libgblap.so) never links, loads or falls back to it.
 *
 * Every function restates one reference function; the citation is given
 * beside each prototype (paths are relative to the LAP source tree).
 * Arithmetic is kept in the reference's exact operation order so that the
 * results are bit-identical to the reference built with gcc -O3 -std=c99
 * (which does not contract a*b+c into FMA); this file must therefore be
 * compiled with -ffp-contract=off on every architecture.
 *
 * Parity pin: tests/golden/ holds fixtures produced by the reference itself
 * (its NOACC objects linked into oracle/_ref/libref.so by oracle/Makefile)
 * plus the two 5x5 fixtures of test_spmv_omp.c / test_tri_solve_omp.c;
 * tests/test_oracle.py checks this restatement against all of them.
 */
#ifndef LAP_ORACLE_H
#define LAP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors pdata (common.h:29-50). */
typedef struct {
  int *lia; int *lja; double *la; int lnnz;
  int *uia; int *uja; double *ua; int unnz;
  double *ichol_vals;
  double *d;
  double *d_r;
  int n;
  double *aux_vec1, *aux_vec2, *aux_vec3;
  const char *prec_op;
  int m, k;
} orc_pdata;

/* BLAS-1 and sparse kernels: simple_blas.c */
double orc_dot(int n, const double *v, const double *w);                 /* simple_blas.c:4-10   */
void   orc_scal(int n, double alpha, double *v);                         /* simple_blas.c:12-16  */
void   orc_axpy(int n, double alpha, const double *x, double *y);        /* simple_blas.c:18-22  */
void   orc_csr_matvec(int n, int nnz, const int *ia, const int *ja,      /* simple_blas.c:24-44  */
                      const double *a, const double *x, double *y,
                      const double *alpha, const double *beta);
void   orc_lower_solve(int n, int nnz, const int *lia, const int *lja,   /* simple_blas.c:46-64  */
                       const double *la, const double *diag,
                       const double *x, double *result);
void   orc_upper_solve(int n, int nnz, const int *uia, const int *uja,   /* simple_blas.c:67-85  */
                       const double *ua, const double *diag,
                       const double *x, double *result);
void   orc_vec_vec(int n, const double *x, const double *y, double *res);/* simple_blas.c:91-95  */
void   orc_vector_reciprocal(int n, const double *v, double *res);       /* simple_blas.c:99-108 */
void   orc_vector_sqrt(int n, const double *v, double *res);             /* simple_blas.c:112-121*/
void   orc_vec_copy(int n, const double *src, double *dest);             /* simple_blas.c:123-128*/
void   orc_vec_zero(int n, double *v);                                   /* simple_blas.c:131-136*/

/* IC(0): factor on the upper CSR (diagonal first in each row), in place,
 * then transpose into the lower CSR (diagonal last).  simple_blas.c:139-182 */
void   orc_ichol_factor(int n, int nnzU, const int *uia, const int *uja, double *ua,
                        const int *lia, const int *lja, double *la);
/* y = (L L^T)^{-1} x.  simple_blas.c:184-223 */
void   orc_ichol_apply(orc_pdata *p, const double *x, double *y);

/* Preconditioners: GS.c, it_jacobi.c, line_jacobi.c; dispatch: prec.c */
void   orc_GS_std(const int *ia, const int *ja, const double *a, int nnzA,   /* GS.c:5-42    */
                  orc_pdata *p, const double *in, double *out);
void   orc_GS_it(const int *ia, const int *ja, const double *a, int nnzA,    /* GS.c:45-92   */
                 orc_pdata *p, const double *in, double *out);
void   orc_GS_it2(const int *ia, const int *ja, const double *a, int nnzA,   /* GS.c:95-159  */
                  orc_pdata *p, const double *in, double *out);
void   orc_it_jacobi(orc_pdata *p, const double *in, double *out);           /* it_jacobi.c:4-33 */
void   orc_line_jacobi(orc_pdata *p, const double *in, double *out);         /* line_jacobi.c:3-7 */
void   orc_prec_function(const int *ia, const int *ja, const double *a,      /* prec.c:6-45  */
                         int nnzA, orc_pdata *p, const double *x, double *y);

/* PCG: cg.c:5-140.  Returns the number of iterations; *flag as the reference
 * (0 converged, 1 maxit).  res_hist needs maxit+2 entries.  true_res (may be
 * NULL) receives ||b - A x|| computed after convergence, as cg.c:113-117
 * prints it.  max_iters_run (<= 0: unlimited) stops early after that many
 * iterations -- used only by the bounded CPU-baseline sample. */
int    orc_cg(int n, int nnz, const int *ia, const int *ja, const double *a,
              double *x, const double *b, double tol, orc_pdata *p, int maxit,
              int *flag, double *res_hist, double *true_res, int max_iters_run);

/* Matrix Market I/O and splitting: io_utils.c.  Arrays are malloc'ed and
 * owned by the caller (free with orc_free). */
typedef struct {
  int n, m, nnz, nnz_unpacked, symmetric;
  int *coo_rows, *coo_cols; double *coo_vals;
  int *csr_ia, *csr_ja; double *csr_vals;
} orc_mmatrix;
int    orc_read_mm(const char *path, orc_mmatrix *A);          /* io_utils.c:15-74   */
int    orc_read_adjacency(const char *path, orc_mmatrix *A);   /* io_utils.c:82-138  */
void   orc_coo_to_csr(orc_mmatrix *A);                         /* io_utils.c:141-235 */
int    orc_read_rhs(const char *path, double *rhs, int n);     /* io_utils.c:239-264 */
/* Strict L, strict U (CSR, columns ascending) and diagonal D.  io_utils.c:268-363 */
void   orc_split(const orc_mmatrix *A, orc_mmatrix *L, orc_mmatrix *U, double *D);
/* Adjacency -> unweighted (weighted=0) or normalised (1) Laplacian, in
 * place on A, then split.  Degrees are accumulated in int as the reference
 * does (io_utils.c:387-395).  io_utils.c:367-491 */
void   orc_create_L_and_split(orc_mmatrix *A, orc_mmatrix *L, orc_mmatrix *U, double *D,
                              int weighted);
/* Insert the diagonal into strict L (last in row) and strict U (first in
 * row), as cg_driver2.c:95-196 does for GS_std on the GPU and ichol on the
 * CPU.  The new arrays replace the old ones. */
void   orc_embed_diagonal(orc_mmatrix *L, orc_mmatrix *U, const double *D);
void   orc_free_matrix(orc_mmatrix *A);
void   orc_free(void *p);

/* One-call CPU solve mirroring cg_driver2.c's NOACC setup (:51-61, :146-196,
 * :354-386) on an in-memory CSR (full symmetric pattern, columns ascending,
 * every diagonal stored).  x must hold x0 on entry.  Returns iterations.
 * setup_s / solve_s (may be NULL) receive wall times. */
int    orc_solve_csr(int n, int nnz, const int *ia, const int *ja, const double *a,
                     const double *b, double *x, const char *prec, double tol,
                     int maxit, int M, int K, int *flag, double *res_hist,
                     double *true_res, int max_iters_run,
                     double *setup_s, double *solve_s);

/* y = M^{-1} x after the same setup (one prec_function call). */
int    orc_prec_apply_csr(int n, int nnz, const int *ia, const int *ja, const double *a,
                          const char *prec, int M, int K, const double *x, double *y);

/* Number of OpenMP threads the multicore mirror uses (1 without OpenMP). */
int    orc_num_threads(void);
int    orc_spmv_threads(void);

#ifdef __cplusplus
}
#endif
#endif
