/* lap_mm_driver.c -- LAP's SpMV benchmark program (mm_driver.c:22-132) on
 * libgblap, printing the same report so LAP's scripts read it unchanged:
 *
 *     lap_mm_driver <matrix.mtx> <n_trials>
 *
 * As mm_driver.c: the matrix is read (here into device CSR by
 * gb_mm_read_csr, the same CSR as read_mm_file + coo_to_csr), x = 1, y = 0,
 * and y = A x runs n_trials times through the csr_matvec surface
 * (cuda_csr_matvec), timed with gettimeofday; the report gives the total and
 * per-call time and ||A x||.  One difference: the timed region ends after the
 * device has finished (gb_synchronize), where LAP's CUDA build stops its
 * clock with the last asynchronous cuSPARSE call still queued. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>

#include "gblap.h"
#include "lap_gblap.h"

int main(int argc, char *argv[]) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s <matrix.mtx> <n_trials>\n", argv[0]);
    return 2;
  }
  const char *matrixFileName = argv[1];
  int n_trials = atoi(argv[2]);
  gb_mm_csr A;
  const int rc = gb_mm_read_csr(matrixFileName, &A);
  if (rc != GB_OK) {
    fprintf(stderr, "lap_mm_driver: cannot read %s: %s\n", matrixFileName, gb_status_str(rc));
    return 1;
  }

  printf("\n\n");
  printf("Matrix info: \n");
  printf("\n");
  printf("\t Matrix size       : %d x %d \n", A.n, A.n);
  printf("\t Matrix nnz        : %d  \n", (int)A.nnz_file);
  printf("\t Matrix nnz un     : %d  \n", A.nnz);
  printf("\t Number of trials  : %d  \n", n_trials);

  double *hx = (double *)malloc(sizeof(double) * (size_t)A.n);
  double *hy = (double *)malloc(sizeof(double) * (size_t)A.n);
  for (int i = 0; i < A.n; ++i) {
    hx[i] = 1.0;
    hy[i] = 0.0;
  }
  double *x = (double *)mallocForDevice(NULL, A.n, sizeof(double));
  double *y = (double *)mallocForDevice(NULL, A.n, sizeof(double));
  memcpyDevice(x, hx, A.n, sizeof(double), (char *)"H2D");
  memcpyDevice(y, hy, A.n, sizeof(double), (char *)"H2D");
  free(hx);
  free(hy);
  double one = 1.0, zero = 0.0;
  initialize_handles();
  initialize_spmv_buffer(A.n, A.nnz, A.ia, A.ja, A.a, x, y, &one, &zero);
  gb_synchronize();

  struct timeval t1, t2;
  gettimeofday(&t1, 0);
  for (int i = 0; i < n_trials; ++i) cuda_csr_matvec(A.n, A.nnz, A.ia, A.ja, A.a, x, y, &one, &zero);
  gb_synchronize();
  gettimeofday(&t2, 0);
  const double time_spmv = (1000000.0 * (t2.tv_sec - t1.tv_sec) + t2.tv_usec - t1.tv_usec) / 1000.0;
  const double time_spmv_seconds = time_spmv / 1000.0;

  printf("\n\n");
  printf("SpMV test summary results: \n");
  printf("\n");
  printf("\t Time (total)        : %2.16f  \n", time_spmv_seconds);
  printf("\t Time (av., per one) : %2.16f  \n", time_spmv_seconds / (double)n_trials);
  printf("\t Norm of A*x         : %16.16e  \n", sqrt(cuda_dot(A.n, y, y)));
  printf("\n\n");
  freeDevice(x);
  freeDevice(y);
  gb_mm_csr_free(&A);
  return 0;
}
