/*
 * lap_gblap.h -- the LAP call surface exported by libgblap.so.
 *
 * These are the C symbols that LAP's CUDA build binds (cuda_blas.h,
 * devMem.h, blas.h, common.h, io_utils.h), with the same names, argument
 * meaning and pointer conventions, so LAP's own drivers and solver sources
 * compiled with -DCUDA=1 link against libgblap.so instead of cuda_blas.o +
 * devMem.o + cuBLAS/cuSPARSE.  Each declaration cites the reference
 * interface it replaces (paths relative to the LAP source tree).
 *
 * Conventions kept from the reference CUDA backend:
 *   - every array argument of the cuda_* / blas.h functions is a DEVICE
 *     pointer (allocate with mallocForDevice); alpha/beta of csr_matvec are
 *     HOST pointers; dot returns a host scalar (it synchronises);
 *   - CSR is 0-based int32 with columns ascending within each row;
 *   - the triangular solves take L / U with the diagonal stored INSIDE the
 *     factor (last entry of each L row, first of each U row) and ignore
 *     `diag`, as cuda_blas.cu:731-820 does;
 *   - initialize_ichol factors IC(0) in place on A's full pattern (the lower
 *     triangle receives L, diagonal included) and cuda_ichol applies
 *     (L L^T)^{-1} reading pdata->ichol_vals with A's ia/ja, as
 *     cuda_blas.cu:261-561 does.
 * Deliberate differences (fixes): memcpyDevice "D2D" is a
 * device-to-device copy; allocation failures are reported on stderr and
 * return NULL; prec_function reports an unknown name on stderr.
 */
#ifndef LAP_GBLAP_H
#define LAP_GBLAP_H

#ifdef __cplusplus
extern "C" {
#endif

/* pdata: identical layout to common.h:29-50 (real_type = double). */
#ifndef LAP_GBLAP_NO_PDATA
typedef struct {
  int *lia;
  int *lja;
  double *la;
  int lnnz;
  int *uia;
  int *uja;
  double *ua;
  int unnz;
  double *ichol_vals;
  double *d;
  double *d_r;
  int n;
  double *aux_vec1, *aux_vec2, *aux_vec3;
  char *prec_op;
  int m, k;
} pdata;

/* mmatrix: identical layout to io_utils.h:26-42. */
typedef struct {
  int *coo_rows;
  int *coo_cols;
  double *coo_vals;
  int *csr_ia;
  int *csr_ja;
  double *csr_vals;
  int n;
  int m;
  int nnz;
  int nnz_unpacked;
  int symmetric;
} mmatrix;
#endif

/* ---- CUDA backend (replaces cuda_blas.h:6-95 / cuda_blas.cu) ---- */
double cuda_dot(const int n, const double *v, const double *w);                    /* cuda_blas.h:6  */
void cuda_scal(const int n, const double alpha, double *v);                        /* cuda_blas.h:8  */
void cuda_axpy(const int n, const double alpha, const double *x, double *y);       /* cuda_blas.h:10 */
void cuda_csr_matvec(const int n, const int nnz, const int *ia, const int *ja,     /* cuda_blas.h:12 */
                     const double *a, const double *x, double *result,
                     const double *al, const double *bet);
void cuda_lower_triangular_solve(const int n, const int nnz, const int *lia,       /* cuda_blas.h:22 */
                                 const int *lja, const double *la, const double *diag,
                                 const double *x, double *result);
void cuda_upper_triangular_solve(const int n, const int nnz, const int *uia,       /* cuda_blas.h:31 */
                                 const int *uja, const double *ua, const double *diag,
                                 const double *x, double *result);
void cuda_vec_vec(const int n, const double *x, const double *y, double *res);     /* cuda_blas.h:40 */
void cuda_vector_sqrt(const int n, const double *v, double *res);                  /* cuda_blas.h:42 */
void cuda_vector_reciprocal(const int n, const double *v, double *res);            /* cuda_blas.h:44 */
void cuda_vec_copy(const int n, const double *src, double *dest);                  /* cuda_blas.h:46 */
void cuda_vec_zero(const int n, double *vec);                                      /* cuda_blas.h:48 */
void initialize_handles(void);                                                     /* cuda_blas.h:50 */
void initialize_spmv_buffer(const int n, const int nnz, int *ia, int *ja,          /* cuda_blas.h:52 */
                            double *a, const double *x, double *result, double *al,
                            double *bet);
void initialize_and_analyze_L_and_U_solve(const int n, const int nnzL, int *lia,   /* cuda_blas.h:63 */
                                          int *lja, double *la, const int nnzU,
                                          int *uia, int *uja, double *ua);
void initialize_L_and_U_descriptors(const int n, const int nnzL, int *lia,         /* cuda_blas.h:73 */
                                    int *lja, double *la, const int nnzU, int *uia,
                                    int *uja, double *ua);
void initialize_ichol(const int n, const int nnzA, int *ia, int *ja, double *a);   /* cuda_blas.h:83 */
void cuda_ichol(const int *ia, const int *ja, double *a, const int nnzA,           /* cuda_blas.h:89 */
                pdata *prec_data, double *x, double *y);

/* ---- device memory layer (replaces devMem.h:2-4 / devMem.cpp) ---- */
void *mallocForDevice(void *x, int n, int size);                                   /* devMem.h:2 */
void memcpyDevice(void *dest, void *src, int n, int size, char *type);             /* devMem.h:3 */
void freeDevice(void *p);                                                          /* devMem.h:4 */

/* ---- backend-neutral BLAS (replaces blas.h:3-48 / blas.c with CUDA=1) ---- */
double dot(const int n, const double *v, const double *w);                         /* blas.h:3  */
void axpy(const int n, const double alpha, double *x, double *y);                  /* blas.h:5  */
void scal(const int n, const double alpha, double *v);                             /* blas.h:7  */
void csr_matvec(const int n, const int nnz, const int *ia, const int *ja,          /* blas.h:9  */
                const double *a, const double *x, double *result, const double *al,
                const double *bet, const char *kind);
void lower_triangular_solve(const int n, const int nnz, const int *lia,            /* blas.h:20 */
                            const int *lja, const double *la, const double *diag,
                            const double *x, double *result);
void upper_triangular_solve(const int n, const int nnz, const int *uia,            /* blas.h:29 */
                            const int *uja, const double *ua, const double *diag,
                            const double *x, double *result);
void ichol(const int *ia, const int *ja, double *a, const int nnzA,                /* blas.h:38 */
           pdata *prec_data, double *x, double *y);
void vec_vec(const int n, const double *x, double *y, double *res);                /* blas.h:40 */
void vector_reciprocal(const int n, const double *v, double *res);                 /* blas.h:42 */
void vector_sqrt(const int n, const double *v, double *res);                       /* blas.h:44 */
void vec_copy(const int n, double *src, double *dest);                             /* blas.h:46 */
void vec_zero(const int n, double *vec);                                           /* blas.h:48 */

/* ---- solver and preconditioners (replaces cg.c, prec.c, GS.c, *jacobi.c) ---- */
/* PCG with cg.c's exact signature and stopping rule (cg.c:5-140): stops when
 * the recursive ||r|| < tol*||r0||, flag 0 = converged, 1 = more than maxit
 * iterations, 2 = breakdown (p'q <= 0 or non-finite; never produced by the
 * reference).  Runs device-resident: no host synchronisation per iteration. */
void cg(int n, double nnz, int *ia, int *ja, double *a, double *x, double *b,     /* common.h:54 */
        double tol, pdata *prec_data, int maxit, int *it, int *flag,
        double *res_norm_history);
void prec_function(int *ia, int *ja, double *a, int nnzA, pdata *prec_data,       /* common.h:52 */
                   double *x, double *y);
void GS_std(int *ia, int *ja, double *a, int nnzA, pdata *prec_data,              /* common.h:70 */
            double *vec_in, double *vec_out);
void GS_it(int *ia, int *ja, double *a, int nnzA, pdata *prec_data,               /* common.h:71 */
           double *vec_in, double *vec_out);
void GS_it2(int *ia, int *ja, double *a, int nnzA, pdata *prec_data,              /* common.h:72 */
            double *vec_in, double *vec_out);
void it_jacobi(int *ia, int *ja, double *a, int nnzA, pdata *prec_data,           /* common.h:73 */
               double *vec_in, double *vec_out);
void line_jacobi(int *ia, int *ja, double *a, int nnzA, pdata *prec_data,         /* common.h:74 */
                 double *vec_in, double *vec_out);

/* ---- Matrix Market I/O (replaces io_utils.h:44-49 / io_utils.c) ---- */
void read_mm_file(const char *matrixFileName, mmatrix *A);                         /* io_utils.h:44 */
void read_adjacency_file(const char *matrixFileName, mmatrix *A);                  /* io_utils.h:45 */
void coo_to_csr(mmatrix *A);                                                       /* io_utils.h:46 */
void read_rhs(const char *rhsFileName, double *rhs);                               /* io_utils.h:47 */
void split(mmatrix *A, mmatrix *L, mmatrix *U, mmatrix *D);                        /* io_utils.h:48 */
void create_L_and_split(mmatrix *A, mmatrix *L, mmatrix *U, mmatrix *D,            /* io_utils.h:49 */
                        int weighted);

#ifdef __cplusplus
}
#endif
#endif
