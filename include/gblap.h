/*
 * gblap.h -- device-resident extended API of libgblap.so (sm_103a).
 *
 * LAP itself has no such layer: its cg() (cg.c:5-140) drives every BLAS call
 * from the host and synchronises three times per iteration.  This API keeps
 * the whole PCG loop on the GPU (fused kernels, device-side convergence
 * test, one CUDA-graph launch per solve) and adds mixed precision, batching
 * and an adjoint.  Plain pointers and sizes only; every array is a DEVICE
 * pointer unless its name ends in _host.  Every function returns a
 * gb_status; results that LAP reports through cg()'s `flag` keep that
 * meaning in gb_pcg_result.flag.
 */
#ifndef GBLAP_H
#define GBLAP_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GB_OK = 0,
  GB_MAXIT = 1,        /* more than maxit iterations (cg.c:119) */
  GB_BREAKDOWN = 2,    /* p'q <= 0 or a non-finite scalar in the recurrence */
  GB_ZERO_PIVOT = 3,   /* IC(0) met a non-positive pivot */
  GB_TIMEOUT = 4,      /* a sync-free wait exceeded its time limit */
  GB_BAD_INPUT = 5,    /* malformed CSR, missing diagonal, bad sizes, unknown name */
  GB_CUDA_ERROR = 6,
  GB_NO_MEMORY = 7,
  GB_NOT_SUPPORTED = 8,
  GB_INTERNAL = 9      /* a device-side consistency check failed (a staged record was not the one expected) */
} gb_status;

/* Preconditioner names are LAP's (prec.c:6-45). */
typedef enum {
  GB_PREC_NONE = 0,        /* "none"        */
  GB_PREC_LINE_JACOBI = 1, /* "line_jacobi" : y = D^-1 x (line_jacobi.c:3-7) */
  GB_PREC_IT_JACOBI = 2,   /* "it_jacobi"   : k Jacobi sweeps (it_jacobi.c:4-33) */
  GB_PREC_GS_STD = 3,      /* "GS_std"      : k forward + k backward GS sweeps (GS.c:5-42) */
  GB_PREC_GS_IT = 4,       /* "GS_it"       : GS.c:45-92 */
  GB_PREC_GS_IT2 = 5,      /* "GS_it2"      : GS.c:95-159 */
  GB_PREC_ICHOL = 6        /* "ichol"       : IC(0) on A's pattern (simple_blas.c:139-223) */
} gb_prec;

const char *gb_status_str(int status);
/* Maps a LAP preconditioner name to gb_prec; returns -1 for an unknown name. */
int gb_prec_from_name(const char *name);
/* Library build string (arch, version). */
const char *gb_version(void);
/* Waits for all device work the calling thread has queued (cudaDeviceSynchronize). */
int gb_synchronize(void);

/* ------------------------------------------------------------ solver object */
typedef struct gb_system_s *gb_system;

/* Wraps a device CSR matrix (full symmetric pattern, 0-based int32 indices,
 * columns ascending, no duplicates, every diagonal stored).  The arrays are
 * borrowed and must outlive the object.  Builds the SpMV row tiling, the
 * level schedules of the triangular factors and, for "ichol", the IC(0)
 * factor on the device.  m, k are LAP's M (outer) and K (inner) counts. */
int gb_system_create(int n, int nnz, const int *ia, const int *ja, const double *a,
                     const char *prec_name, int m, int k, gb_system *out);
int gb_system_destroy(gb_system sys);
/* Re-reads the matrix values (same pattern) and refactors / refreshes the
 * preconditioner and the FP32 copies. */
int gb_system_update_values(gb_system sys);
/* Re-reads only the matrix values (same pattern) into the system's derived
 * arrays: the FP32 copy, the diagonal and its reciprocal.  The
 * preconditioner's values are left as they are. */
int gb_system_refresh_matrix(gb_system sys);
/* Loads the preconditioner's values from caller-owned device arrays laid
 * out as LAP's pdata holds them (common.h:29-50), instead of deriving them
 * from A -- what LAP's cg() applies through prec_function (prec.c:6-45):
 *   line_jacobi                d_r = 1/diag (line_jacobi.c:3-7);
 *   it_jacobi, GS_it, GS_it2   strict L (lia, lja, la, lnnz) and U, and d_r
 *                              (it_jacobi.c:4-33, GS.c:45-159);
 *   GS_std                     L with its diagonal last in each row and U
 *                              with it first, as cg_driver2.c:95-144 builds
 *                              them (GS.c:5-42);
 *   ichol                      ichol_vals: the IC(0) factor on A's pattern
 *                              with L in the lower triangle, as
 *                              initialize_ichol leaves it (cuda_blas.cu:490-561).
 * Unused arguments may be NULL.  L / U layouts must be the ones LAP's driver
 * derives from this system's A (checked by pattern fingerprint; GB_BAD_INPUT
 * otherwise). */
int gb_system_set_prec_values(gb_system sys, const int *lia, const int *lja, const double *la, int lnnz,
                              const int *uia, const int *uja, const double *ua, int unnz,
                              const double *d_r, const double *ichol_vals);
/* Fingerprint of a device CSR pattern (ia [n+1], ja [nnz]): a 64-bit sum of
 * mixed (position, value) pairs, order-independent.  Caches keyed by array
 * addresses compare it to notice new contents behind an old address.
 * Synchronises the system's stream. */
int gb_system_pattern_hash(gb_system sys, int n, int nnz, const int *ia, const int *ja,
                           unsigned long long *out);
/* Levels of the lower / upper sync-free schedules and SpMV tiles (diagnostics). */
int gb_system_info(gb_system sys, int *lower_levels, int *upper_levels, int *spmv_tiles);

typedef struct {
  double tol;        /* stop when ||r|| < tol*||r0|| (cg.c:60,107); mixed: ||b-Ax|| < tol*||b-Ax0|| */
  int maxit;         /* iteration cap; like cg.c at most maxit+1 iterations run */
  int precision;     /* 0: FP64 PCG.
                        1: FP32 inner PCG (FP32 Krylov vectors, SpMV and preconditioner)
                           inside FP64 iterative refinement.
                        2: split: FP64 Krylov vectors and scalars around an FP32 SpMV and
                           FP32 triangular-solve preconditioner ("ichol", "GS_std" with
                           k = 1), with FP64 residual replacement.
                        -1 (gb_pcg_solve, gb_pcg_solve_host): the mode
                           gb_pcg_autotune_precision chose for the system (0 until it
                           has run).  */
  double inner_tol;  /* mixed: residual reduction between refinement / replacement steps;
                        0 (default) selects 1e-4 for precision 1 and 1e-2 for precision 2.
                        A cycle never runs past the solve's own tolerance. */
  int max_outer;     /* mixed: refinement steps cap (default 50) */
  int use_graph;     /* 1 (default): the iteration loop is one CUDA graph with a device-side
                        while node; 0: host-launched kernels, one status read per 16 iterations */
  int verbose;       /* print LAP's per-iteration line "CG: it %d, res norm %5.5e" */
} gb_pcg_opts;

typedef struct {
  int iters;           /* PCG iterations (mixed: sum over refinement steps) */
  int outer;           /* refinement steps (mixed), 0 for FP64 */
  int flag;            /* cg.c: 0 converged, 1 maxit, 2 failure */
  int status;          /* gb_status */
  double res0;         /* ||b - A x0|| */
  double res;          /* final recursive residual norm (FP64 true residual for mixed) */
  double true_res;     /* ||b - A x|| recomputed in FP64 after the solve */
  double rel_true_res; /* true_res / ||b|| (the quantity cg.c:117 prints) */
  double device_ms;    /* device time of the solve, CUDA events on the system stream */
} gb_pcg_result;

void gb_pcg_opts_default(gb_pcg_opts *opts);

/* Solves A x = b.  x holds x0 on entry.  res_hist_host (may be NULL) receives
 * up to hist_len residual norms, res_hist_host[0] = ||r0|| as cg.c.  Blocks
 * until the solve is complete. */
int gb_pcg_solve(gb_system sys, const double *b, double *x, const gb_pcg_opts *opts,
                 double *res_hist_host, int hist_len, gb_pcg_result *result);

/* Same solve, from and to HOST buffers (b_host, x_host of n doubles; x_host
 * holds x0).  The host<->device copies are part of the call. */
int gb_pcg_solve_host(gb_system sys, const double *b_host, double *x_host,
                      const gb_pcg_opts *opts, gb_pcg_result *result);

/* ------------------------------------------------------------ kernels */
/* y = alpha*A*x + beta*y (FP64), LAP's row-sequential summation order. */
int gb_spmv(gb_system sys, double alpha, const double *x, double beta, double *y);
/* y = M^{-1} x with the system's preconditioner (prec_function semantics). */
int gb_precond_apply(gb_system sys, const double *x, double *y);
/* IC(0) factor values in LAP's CPU layout: L (diagonal last per row, strict
 * lower pattern + diagonal) and U = L^T (diagonal first), each nnz_lower+n
 * doubles, device pointers. */
int gb_ichol_factor_values(gb_system sys, double *l_vals, double *u_vals);

/* ------------------------------------------------------------ adjoint */
/* Given the solution x of A x = b and the adjoint lambda of A lambda = g,
 * writes G[k] = -lambda[i] * x[j] for every stored entry k = (i, j) of A
 * (dL/dA on A's pattern) and, when edge_grad is non-NULL, for every entry of
 * the strict lower triangle in row-major order the edge-weight gradient
 * dL/dw_ij = G_ij + G_ji - G_ii - G_jj = -(lambda_i - lambda_j)(x_i - x_j)
 * for a Laplacian A = L(w) + shift. */
int gb_adjoint_scatter(gb_system sys, const double *x, const double *lambda, double *G,
                       double *edge_grad);
/* Full adjoint step: solves A lambda = g with the same PCG (A is SPD) and
 * scatters.  dL/db = lambda. */
int gb_adjoint_grad(gb_system sys, const double *x, const double *g, double *lambda,
                    double *G, double *edge_grad, const gb_pcg_opts *opts,
                    gb_pcg_result *result);

/* ------------------------------------------------------------ batching */
typedef struct gb_batch_s *gb_batch;
/* count independent CSR systems concatenated block-diagonally (device arrays):
 * ia holds the N+1 row pointers of the concatenation (N = row_off[count]),
 * ja each entry's column index LOCAL to its system (0-based), a the values.
 * row_off[count+1] and nnz_off[count+1] (host, int64) give each system's
 * first row and first entry; ia[row_off[s]] must equal nnz_off[s].  Every
 * row needs a nonzero diagonal.  Preconditioner: "line_jacobi" or "none".
 * The arrays are borrowed and must outlive the batch. */
int gb_batch_create(int count, const long long *row_off_host, const long long *nnz_off_host,
                    const int *ia, const int *ja, const double *a, const char *prec_name,
                    gb_batch *out);
int gb_batch_destroy(gb_batch batch);
/* Solves every system in one persistent launch (a CUDA graph whose while
 * node runs until every system stopped); b, x concatenated [N], x holds x0.
 * opts->precision 0 (FP64) or 2 (FP32 matrix values and products inside the
 * FP64 recurrence with per-system residual replacement).  iters_host /
 * flags_host (may be NULL) receive per-system iteration counts and cg.c
 * flags; result aggregates them (maximum iterations, worst flag, largest
 * true residual). */
int gb_batch_solve(gb_batch batch, const double *b, double *x, const gb_pcg_opts *opts,
                   int *iters_host, int *flags_host, gb_pcg_result *result);

/* Multi-RHS: nrhs right-hand sides on one system, B and X row-major
 * [nrhs][n] (X holds x0).  Each column runs its own PCG recurrence in the
 * batch engine above; up to 32 columns share one read of the matrix per
 * iteration (more run as consecutive chunks of 32 and a shorter last one;
 * iters_host still receives every column's count and result aggregates
 * all columns, device_ms summed over the chunks).  Systems with
 * "line_jacobi" or "none"; precision 0 or 2. */
int gb_pcg_solve_multi(gb_system sys, int nrhs, const double *B, double *X,
                       const gb_pcg_opts *opts, int *iters_host, gb_pcg_result *result);

/* ------------------------------------------------------------ autotuner */
/* Times the SpMV variants on this system and keeps the fastest (cached per
 * matrix shape class).  best_host receives the chosen rows-per-bundle. */
int gb_autotune_spmv(gb_system sys, int *best_host);

/* Picks a block-diagonal batch's row-bundle and tile sizes by timing them:
 * rows per SpMV bundle in {32, 16, 8} x rows per update / reduction chunk in
 * {2048, 1024, 4096}, each running `iters` iterations (<= 0: 16) of the
 * batch's own captured solve loop (FP64, no stopping) on right-hand side b;
 * the fastest is applied to the batch and cached per matrix class (system
 * count, rows, entries, longest row), so later batches of that class are set
 * without timing.  Results of the tuned batch equal the default's up to the
 * rounding of the regrouped reductions.  Outputs may be NULL; the times are
 * 0 when the choice came from the cache.  GB_NOT_SUPPORTED for multi-RHS
 * batches (see gb_pcg_autotune_multi).  No counterpart in LAP. */
int gb_batch_autotune(gb_batch batch, const double *b, int iters, int *rows_per_bundle, int *chunk_rows,
                      double *ms_default, double *ms_best);

/* Picks the columns per interleaved chunk of gb_pcg_solve_multi for nrhs
 * right-hand sides B ([nrhs][n], device) on this system by timing 32, 16 and
 * 8 over `iters` iterations; the fastest is kept on the system (and cached
 * per (n, nnz, nrhs)).  No counterpart in LAP. */
int gb_pcg_autotune_multi(gb_system sys, int nrhs, const double *B, int iters, int *width, double *ms_default,
                          double *ms_best);

/* Picks the precision mode of the system's solves by timing: one solve of b
 * (device, x0 = 0) with *opts in each mode 0, 1, 2 that the system supports,
 * each timed on its second run (the first also captures the mode's graph and
 * fills its FP32 records).  The fastest that converged is kept on the system
 * (used by precision = -1) and returned in *best; ms_host[3] (may be NULL)
 * receives each mode's device time, -1 where the mode is unsupported or did
 * not converge.  GB_MAXIT when no mode converged.  No counterpart in LAP. */
int gb_pcg_autotune_precision(gb_system sys, const double *b, const gb_pcg_opts *opts, int *best,
                              double *ms_host);

/* ------------------------------------------------------------ failure injection */
/* Test hook: wall-clock limit (ns) of every sync-free wait in this system's
 * solves and factorization; 0 restores the default of one second.  A wait
 * that runs out records GB_TIMEOUT, releases its dependents with a NaN and
 * returns, so the solve ends with status GB_TIMEOUT instead of hanging. */
int gb_debug_set_spin_budget(gb_system sys, unsigned long long ns);

/* ------------------------------------------------------------ measurement */
/* Per-kernel device times (ms per launch, CUDA events on the system stream)
 * of one PCG iteration's kernels, averaged over `iters` iterations run
 * eagerly.  names_host receives a ';'-separated list of kernel names,
 * ms_host[i] and bytes_host[i] the average time and algorithmic bytes. */
int gb_profile_iteration(gb_system sys, const double *b, double *x, int precision, int iters,
                         char *names_host, int names_len, double *ms_host,
                         double *bytes_host, int max_kernels, int *count);

/* ------------------------------------------------------------ allocation-free dot */
/* Largest n gb_dot_noalloc accepts (8192 partials of 4096 elements). */
#define GB_DOT_NOALLOC_MAX_N 33554432

/* *result_host = v'w for device vectors v, w of length n, without allocating
 * any device memory.  No counterpart in LAP, whose dot() (cuda_blas.cu via
 * blas.h) works in cuBLAS-owned memory; this library's cuda_dot()
 * allocates its scratch on first use.  For callers that cannot let a
 * library allocate: processes whose device memory is already claimed by
 * another allocator (a late cudaMalloc would fail), and loops that must not
 * risk the implicit synchronisation of cudaMalloc / cudaFree while other
 * streams have work in flight.  The scratch (partials, completion ticket,
 * result) lives in one fixed 64 KB array per device inside this library.
 *   - n > GB_DOT_NOALLOC_MAX_N is rejected with GB_BAD_INPUT (and a message
 *     on stderr) before any device work; use cuda_dot() for longer vectors.
 *   - The first call on each device, with that device current, sets up the
 *     scratch address (cudaGetSymbolAddress); make it before any stream
 *     capture begins.
 *   - Calls that can overlap on one device (several host threads, or
 *     unordered streams) share the scratch and race: serialise them.
 * stream: a cudaStream_t, or NULL for the legacy default stream.  Every
 * call blocks: it ends with a copy of the result into *result_host and
 * waits for the stream, so it returns with the sum in hand.  The rounding
 * depends on n only (fixed chunking), and may differ from cuda_dot() in the
 * last bits. */
int gb_dot_noalloc(int n, const double *v, const double *w, double *result_host, void *stream);

/* ------------------------------------------------------------ Matrix Market on the device */
/* A CSR matrix built on the device from a Matrix Market coordinate file.
 * ia [n+1], ja [nnz], a [nnz] are device arrays owned by the caller (free
 * them with gb_mm_csr_free). */
typedef struct {
  int n, m;              /* rows, columns (size line) */
  long long nnz_file;    /* entries the size line announces */
  int nnz;               /* CSR entries: a symmetric file's off-diagonal entries mirrored */
  int symmetric, pattern;
  int *ia, *ja;
  double *a;
  int host_parsed;       /* values outside the device's exact decimal path, parsed by strtod */
  double read_ms;        /* gb_mm_read_csr: the file read, with the copy to the device overlapped */
  double h2d_ms;         /* gb_mm_parse_csr: the bytes' copy to the device (0 for a file) */
  double device_ms;      /* line split, parse, mirror, sort and CSR build */
} gb_mm_csr;

/* read_mm_file (io_utils.c:15-74) followed by coo_to_csr (io_utils.c:141-235),
 * with the same CSR bit for bit, built on the device: the host reads the
 * header, reader threads read the rest in 4 MB chunks and copy each to the
 * device while reading the next (GBLAP_MM_READ_THREADS, default 8), and
 * line splitting, number
 * parsing (values rounded to the nearest double exactly, as strtod does),
 * symmetric mirroring and the column sort run as device kernels.  Lines
 * starting with '%' and blank lines are skipped; entries past the size line's
 * count are ignored.  GB_BAD_INPUT for a missing size line, a malformed or
 * out-of-range entry, or fewer entries than announced; GB_NOT_SUPPORTED for
 * sizes past int32. */
int gb_mm_read_csr(const char *path, gb_mm_csr *out);
/* The same from the whole file held in host memory. */
int gb_mm_parse_csr(const char *bytes, long long len, gb_mm_csr *out);
int gb_mm_csr_free(gb_mm_csr *m);

/* The Laplacian driver's setup (cg_driver.c:38-45) on the device:
 * read_adjacency_file (io_utils.c:82-138: the file's entries, symmetric
 * whatever the banner says, plus one unit diagonal entry per vertex),
 * coo_to_csr, then create_L_and_split's in-place Laplacian
 * (io_utils.c:367-491): weighted = 0 gives D - W, weighted = 1 gives
 * I - D^-1/2 W D^-1/2.  The reference sums each degree into an int, so
 * every partial sum of a non-integer weight is truncated toward zero
 * (io_utils.c:387-395); exact_degrees = 0 reproduces that, 1 sums in double.
 * out->a holds the Laplacian's values on A's pattern. */
int gb_mm_read_laplacian(const char *path, int weighted, int exact_degrees, gb_mm_csr *out);
int gb_mm_parse_laplacian(const char *bytes, long long len, int weighted, int exact_degrees,
                          gb_mm_csr *out);
/* The driver's right-hand side (cg_driver.c:159-230): b_i = (-1)^i, minus
 * its component along the null vector e/sqrt(n) (weighted = 0) or
 * sqrt(d)/||sqrt(d)|| (weighted = 1, d the Laplacian's diagonal, read from
 * ia/ja/a), with LAP's BLAS-1 call sequence on the legacy default stream.
 * b: device [n] (output); work: device scratch [n]. */
int gb_laplacian_rhs(int n, const int *ia, const int *ja, const double *a, int weighted, double *b,
                     double *work);

#ifdef __cplusplus
}
#endif
#endif
