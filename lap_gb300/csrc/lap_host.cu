// lap_host.cu -- LAP's solver-level C surface: cg() (cg.c), prec_function()
// and the preconditioners (prec.c, GS.c, it_jacobi.c, line_jacobi.c) and the
// Matrix Market I/O (io_utils.c), written for the GPU build.
//
// cg() keeps the reference's signature, stopping rule, flag values and
// residual history, but runs the device-resident engine (gb_pcg_solve): no
// host synchronisation per iteration.  The engine object for a matrix is
// cached by (ia, ja, a, sizes, preconditioner) and revalidated on every call
// by the fingerprint of (ia, ja), so its analysis (SpMV tiling, level
// schedules) is reused while the pattern is the same and rebuilt when new
// contents sit behind the same addresses.  Values are never taken from the
// cache: each call re-reads A's values and applies the preconditioner data
// pdata holds -- d_r, la / ua, ichol_vals -- as LAP's prec_function does.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "gblap.h"
#include "lap_gblap.h"

namespace {

struct SysKey {
  const void *ia, *ja, *a;
  int n, nnz, m, k;
  std::string prec;
  bool operator<(const SysKey& o) const {
    return std::tie(ia, ja, a, n, nnz, m, k, prec) < std::tie(o.ia, o.ja, o.a, o.n, o.nnz, o.m, o.k, o.prec);
  }
};

struct SysEntry {
  gb_system sys = nullptr;
  unsigned long long pattern = 0;
};

std::mutex g_sys_mu;
auto& g_systems = *new std::map<SysKey, SysEntry>;  // never destroyed: no CUDA calls at exit

// The preconditioner values LAP's cg() would apply: pdata's arrays where the
// preconditioner reads them, else (arrays not set) derived from A.
int load_prec_data(gb_system sys, const pdata* p) {
  const int prec = gb_prec_from_name(p->prec_op);
  const bool have = prec == GB_PREC_NONE ||
                    (prec == GB_PREC_LINE_JACOBI && p->d_r) ||
                    (prec == GB_PREC_ICHOL && p->ichol_vals) ||
                    (prec == GB_PREC_GS_STD && p->lia && p->la && p->uia && p->ua) ||
                    ((prec == GB_PREC_IT_JACOBI || prec == GB_PREC_GS_IT || prec == GB_PREC_GS_IT2) &&
                     p->lia && p->la && p->uia && p->ua && p->d_r);
  if (!have) return gb_system_update_values(sys);
  const int rc = gb_system_refresh_matrix(sys);
  if (rc != GB_OK) return rc;
  return gb_system_set_prec_values(sys, p->lia, p->lja, p->la, p->lnnz, p->uia, p->uja, p->ua, p->unnz,
                                   p->d_r, p->ichol_vals);
}

bool verbose() {
  const char* v = getenv("GBLAP_VERBOSE");
  return v && v[0] && v[0] != '0';
}

}  // namespace

// ============================================================ cg.c
extern "C" void cg(int n, double nnz, int* ia, int* ja, double* a, double* x, double* b, double tol,
                   pdata* prec_data, int maxit, int* it, int* flag, double* res_norm_history) {
  const int innz = (int)nnz;
  *it = 0;
  *flag = 2;
  if (gb_prec_from_name(prec_data->prec_op) < 0) {
    fprintf(stderr, "libgblap: cg: unknown preconditioner '%s' (prec.c accepts it_jacobi, "
                    "line_jacobi, GS_std, GS_it, ichol, GS_it2, none)\n", prec_data->prec_op);
    return;
  }
  gb_system sys = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_sys_mu);
    SysKey key{ia, ja, a, n, innz, prec_data->m, prec_data->k, prec_data->prec_op};
    auto f = g_systems.find(key);
    if (f != g_systems.end()) {
      unsigned long long h = 0;
      const int rc = gb_system_pattern_hash(f->second.sys, n, innz, ia, ja, &h);
      if (rc == GB_OK && h == f->second.pattern) {
        sys = f->second.sys;
      } else {  // another pattern behind the same addresses: rebuild
        gb_system_destroy(f->second.sys);
        g_systems.erase(f);
      }
    }
    if (!sys) {
      int rc = gb_system_create(n, innz, ia, ja, a, prec_data->prec_op, prec_data->m, prec_data->k, &sys);
      SysEntry e;
      e.sys = sys;
      if (rc == GB_OK) rc = gb_system_pattern_hash(sys, n, innz, ia, ja, &e.pattern);
      if (rc != GB_OK) {
        if (sys) gb_system_destroy(sys);
        fprintf(stderr, "libgblap: cg: setup failed: %s\n", gb_status_str(rc));
        return;
      }
      g_systems[key] = e;
    }
    const int rc = load_prec_data(sys, prec_data);
    if (rc != GB_OK) {
      fprintf(stderr, "libgblap: cg: preconditioner data (pdata) for '%s' does not match A: %s\n",
              prec_data->prec_op, gb_status_str(rc));
      return;
    }
  }
  gb_pcg_opts o;
  gb_pcg_opts_default(&o);
  o.tol = tol;
  o.maxit = maxit;
  gb_pcg_result r;
  const int rc = gb_pcg_solve(sys, b, x, &o, res_norm_history, maxit + 2, &r);
  if (rc != GB_OK) fprintf(stderr, "libgblap: cg: %s\n", gb_status_str(rc));
  *it = r.iters;
  *flag = r.flag;
  if (verbose())
    for (int i = 0; i <= r.iters && i <= maxit + 1; ++i)
      printf("CG: it %d, res norm %5.5e \n", i, res_norm_history[i]);
  if (r.flag == 0)
    printf("TRUE Norm of r %5.5e relative %16.16e\n", r.true_res, r.rel_true_res);
}

// ============================================================ preconditioners
// GS.c:5-42 with LAP's GPU convention (diagonal inside L and U).
extern "C" void GS_std(int* ia, int* ja, double* a, int nnzA, pdata* p, double* vin, double* vout) {
  const int n = p->n;
  const double one = 1.0, minusone = -1.0;
  vec_zero(n, vout);
  for (int i = 0; i < p->k; ++i) {
    vec_copy(n, vin, p->aux_vec2);
    csr_matvec(n, nnzA, ia, ja, a, vout, p->aux_vec2, &minusone, &one, "A");
    lower_triangular_solve(n, p->lnnz, p->lia, p->lja, p->la, p->d, p->aux_vec2, p->aux_vec1);
    axpy(n, 1.0, p->aux_vec1, vout);
  }
  for (int i = 0; i < p->k; ++i) {
    vec_copy(n, vin, p->aux_vec2);
    csr_matvec(n, nnzA, ia, ja, a, vout, p->aux_vec2, &minusone, &one, "A");
    upper_triangular_solve(n, p->unnz, p->uia, p->uja, p->ua, p->d, p->aux_vec2, p->aux_vec1);
    axpy(n, 1.0, p->aux_vec1, vout);
  }
}

// GS.c:45-92
extern "C" void GS_it(int* ia, int* ja, double* a, int nnzA, pdata* p, double* vin, double* vout) {
  const int n = p->n;
  const double one = 1.0, minusone = -1.0;
  vec_zero(n, vout);
  for (int j = 0; j < p->m; ++j) {
    vec_copy(n, vin, p->aux_vec2);
    csr_matvec(n, nnzA, ia, ja, a, vout, p->aux_vec2, &minusone, &one, "A");
    vec_vec(n, p->aux_vec2, p->d_r, p->aux_vec1);
    for (int i = 0; i < p->k; ++i) {
      vec_copy(n, p->aux_vec2, p->aux_vec3);
      csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, p->aux_vec1, p->aux_vec3, &minusone, &one, "L");
      vec_vec(n, p->aux_vec3, p->d_r, p->aux_vec1);
    }
    for (int i = 0; i < p->k; ++i) {
      vec_copy(n, p->aux_vec2, p->aux_vec3);
      csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, p->aux_vec1, p->aux_vec3, &minusone, &one, "U");
      vec_vec(n, p->aux_vec3, p->d_r, p->aux_vec1);
    }
    axpy(n, 1.0, p->aux_vec1, vout);
  }
}

// GS.c:95-159
extern "C" void GS_it2(int* ia, int* ja, double* a, int nnzA, pdata* p, double* vin, double* vout) {
  (void)ia; (void)ja; (void)a; (void)nnzA;
  const int n = p->n;
  const double one = 1.0, zero = 0.0, minusone = -1.0;
  double *v1 = p->aux_vec1, *v2 = p->aux_vec2, *v3 = p->aux_vec3;
  vec_vec(n, vin, p->d_r, v1);
  for (int j = 0; j < p->m; ++j) {
    csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, v1, v2, &one, &zero, "L");
    csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, v1, v3, &one, &zero, "U");
    axpy(n, 1.0, v3, v2);
    vec_copy(n, vin, v3);
    axpy(n, -1.0, v2, v3);
    vec_vec(n, v3, p->d_r, v2);
    vec_copy(n, vin, v3);
    csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, v2, v3, &minusone, &one, "L");
    for (int i = 0; i < p->k; ++i) {
      vec_copy(n, v3, v1);
      csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, v2, v1, &minusone, &one, "U");
      vec_vec(n, p->d_r, v1, v2);
    }
    vec_copy(n, vin, v3);
    csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, v2, v3, &minusone, &one, "U");
    for (int i = 0; i < p->k; ++i) {
      vec_copy(n, v3, v1);
      csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, v2, v1, &minusone, &one, "L");
      vec_vec(n, p->d_r, v1, v2);
    }
    vec_copy(n, v2, v1);
  }
  vec_copy(n, v2, vout);
}

// it_jacobi.c:4-33
extern "C" void it_jacobi(int* ia, int* ja, double* a, int nnzA, pdata* p, double* vin, double* vout) {
  (void)ia; (void)ja; (void)a; (void)nnzA;
  const int n = p->n;
  const double one = 1.0, zero = 0.0;
  vec_zero(n, vout);
  for (int i = 0; i < p->k; ++i) {
    csr_matvec(n, p->lnnz, p->lia, p->lja, p->la, vout, p->aux_vec1, &one, &zero, "L");
    csr_matvec(n, p->unnz, p->uia, p->uja, p->ua, vout, p->aux_vec2, &one, &zero, "U");
    axpy(n, 1.0, p->aux_vec1, p->aux_vec2);
    vec_copy(n, vin, vout);
    axpy(n, -1.0, p->aux_vec2, vout);
    vec_vec(n, vout, p->d_r, vout);
  }
}

// line_jacobi.c:3-7
extern "C" void line_jacobi(int* ia, int* ja, double* a, int nnzA, pdata* p, double* vin, double* vout) {
  (void)ia; (void)ja; (void)a; (void)nnzA;
  vec_vec(p->n, p->d_r, vin, vout);
}

// prec.c:6-45; an unknown name is reported instead of silently skipped
extern "C" void prec_function(int* ia, int* ja, double* a, int nnzA, pdata* p, double* x, double* y) {
  const char* op = p->prec_op;
  if (strcmp(op, "it_jacobi") == 0) it_jacobi(ia, ja, a, nnzA, p, x, y);
  else if (strcmp(op, "line_jacobi") == 0) line_jacobi(ia, ja, a, nnzA, p, x, y);
  else if (strcmp(op, "GS_std") == 0) GS_std(ia, ja, a, nnzA, p, x, y);
  else if (strcmp(op, "GS_it") == 0) GS_it(ia, ja, a, nnzA, p, x, y);
  else if (strcmp(op, "ichol") == 0) ichol(ia, ja, a, nnzA, p, x, y);
  else if (strcmp(op, "GS_it2") == 0) GS_it2(ia, ja, a, nnzA, p, x, y);
  else if (strcmp(op, "none") == 0) vec_copy(p->n, x, y);
  else fprintf(stderr, "libgblap: prec_function: unknown preconditioner '%s'\n", op);
}

// ============================================================ io_utils.c
namespace {

// Reads the banner and skips comment lines; returns the size line.
bool mm_header(FILE* f, std::string* banner, char* line, size_t len) {
  if (!fgets(line, (int)len, f)) return false;
  *banner = line;
  while (line[0] == '%')
    if (!fgets(line, (int)len, f)) return false;
  return true;
}

void mm_read_entries(FILE* f, bool pattern, int count, mmatrix* A) {
  char line[256];
  int i = 0;
  while (i < count && fgets(line, sizeof line, f)) {
    if (line[0] == '%' || line[0] == '\n') continue;
    int r = 0, c = 0;
    double v = 1.0;
    const int got = pattern ? sscanf(line, "%d %d", &r, &c) : sscanf(line, "%d %d %lf", &r, &c, &v);
    if (got < 2) continue;
    if (r < 1 || c < 1) fprintf(stderr, "libgblap: read_mm_file: bad index %d %d\n", r, c);
    A->coo_rows[i] = r - 1;
    A->coo_cols[i] = c - 1;
    A->coo_vals[i] = v;
    ++i;
  }
  if (i != count) fprintf(stderr, "libgblap: Matrix Market file ended after %d of %d entries\n", i, count);
}

}  // namespace

// io_utils.c:15-74: coordinate format; 'pattern' -> values 1.0; 'symmetric'
// recorded for coo_to_csr; indices converted to 0-based.
extern "C" void read_mm_file(const char* path, mmatrix* A) {
  memset(A, 0, sizeof(*A));
  FILE* f = fopen(path, "r");
  if (!f) {
    fprintf(stderr, "libgblap: read_mm_file: cannot open %s\n", path);
    return;
  }
  char line[256];
  std::string banner;
  if (!mm_header(f, &banner, line, sizeof line)) {
    fclose(f);
    return;
  }
  const bool pattern = banner.find("pattern") != std::string::npos;
  A->symmetric = banner.find("symmetric") != std::string::npos;
  long n = 0, m = 0, nnz = 0;
  sscanf(line, "%ld %ld %ld", &n, &m, &nnz);
  A->n = (int)n;
  A->m = (int)m;
  A->nnz = (int)nnz;
  A->coo_rows = (int*)calloc((size_t)nnz + 1, sizeof(int));
  A->coo_cols = (int*)calloc((size_t)nnz + 1, sizeof(int));
  A->coo_vals = (double*)calloc((size_t)nnz + 1, sizeof(double));
  mm_read_entries(f, pattern, (int)nnz, A);
  fclose(f);
}

// io_utils.c:82-138: adjacency, plus one unit diagonal entry per vertex
// (replaced by the degree in create_L_and_split).
extern "C" void read_adjacency_file(const char* path, mmatrix* A) {
  memset(A, 0, sizeof(*A));
  FILE* f = fopen(path, "r");
  if (!f) {
    fprintf(stderr, "libgblap: read_adjacency_file: cannot open %s\n", path);
    return;
  }
  char line[256];
  std::string banner;
  if (!mm_header(f, &banner, line, sizeof line)) {
    fclose(f);
    return;
  }
  const bool pattern = banner.find("pattern") != std::string::npos;
  A->symmetric = 1;
  long n = 0, m = 0, nnz = 0;
  sscanf(line, "%ld %ld %ld", &n, &m, &nnz);
  A->n = (int)n;
  A->m = (int)m;
  A->nnz = (int)nnz;
  A->coo_rows = (int*)calloc((size_t)(nnz + n) + 1, sizeof(int));
  A->coo_cols = (int*)calloc((size_t)(nnz + n) + 1, sizeof(int));
  A->coo_vals = (double*)calloc((size_t)(nnz + n) + 1, sizeof(double));
  mm_read_entries(f, pattern, (int)nnz, A);
  fclose(f);
  for (int j = 0; j < A->n; ++j) {
    A->coo_rows[nnz + j] = j;
    A->coo_cols[nnz + j] = j;
    A->coo_vals[nnz + j] = 1.0;
  }
  A->nnz += A->n;
}

// io_utils.c:141-235: COO -> CSR; a symmetric matrix's off-diagonal entries
// are mirrored; columns ascending within a row; duplicates are kept (not
// merged), in input order.
extern "C" void coo_to_csr(mmatrix* A) {
  const int n = A->n;
  std::vector<int> cnt(n + 1, 0);
  long total = 0;
  for (int i = 0; i < A->nnz; ++i) {
    cnt[A->coo_rows[i]]++;
    ++total;
    if (A->symmetric && A->coo_rows[i] != A->coo_cols[i]) {
      cnt[A->coo_cols[i]]++;
      ++total;
    }
  }
  A->nnz_unpacked = (int)total;
  A->csr_ia = (int*)calloc((size_t)n + 1, sizeof(int));
  A->csr_ja = (int*)calloc((size_t)total + 1, sizeof(int));
  A->csr_vals = (double*)calloc((size_t)total + 1, sizeof(double));
  for (int i = 0; i < n; ++i) A->csr_ia[i + 1] = A->csr_ia[i] + cnt[i];
  std::vector<int> fill(A->csr_ia, A->csr_ia + n);
  for (int i = 0; i < A->nnz; ++i) {
    const int r = A->coo_rows[i], c = A->coo_cols[i];
    const double v = A->coo_vals[i];
    int p = fill[r]++;
    A->csr_ja[p] = c;
    A->csr_vals[p] = v;
    if (A->symmetric && r != c) {
      p = fill[c]++;
      A->csr_ja[p] = r;
      A->csr_vals[p] = v;
    }
  }
  std::vector<std::pair<int, double>> row;
  for (int i = 0; i < n; ++i) {
    const int b = A->csr_ia[i], e = A->csr_ia[i + 1];
    row.clear();
    for (int k = b; k < e; ++k) row.emplace_back(A->csr_ja[k], A->csr_vals[k]);
    std::stable_sort(row.begin(), row.end(),
                     [](const std::pair<int, double>& x, const std::pair<int, double>& y) { return x.first < y.first; });
    for (int k = b; k < e; ++k) {
      A->csr_ja[k] = row[k - b].first;
      A->csr_vals[k] = row[k - b].second;
    }
  }
  free(A->coo_rows);
  free(A->coo_cols);
  free(A->coo_vals);
  A->coo_rows = A->coo_cols = nullptr;
  A->coo_vals = nullptr;
}

// io_utils.c:239-264: the first column of an MM array file.
extern "C" void read_rhs(const char* path, double* rhs) {
  FILE* f = fopen(path, "r");
  if (!f) {
    fprintf(stderr, "libgblap: read_rhs: cannot open %s\n", path);
    return;
  }
  char line[256];
  std::string banner;
  if (!mm_header(f, &banner, line, sizeof line)) {
    fclose(f);
    return;
  }
  long N = 0, m = 0;
  sscanf(line, "%ld %ld", &N, &m);
  long i = 0;
  while (i < N && fgets(line, sizeof line, f)) {
    double v = 0.0;
    if (sscanf(line, "%lf", &v) == 1) rhs[i++] = v;
  }
  fclose(f);
}

namespace {
void alloc_csr(mmatrix* M, int n, int nnz) {
  M->csr_ia = (int*)calloc((size_t)n + 1, sizeof(int));
  M->csr_ja = (int*)calloc((size_t)nnz + 1, sizeof(int));
  M->csr_vals = (double*)calloc((size_t)nnz + 1, sizeof(double));
}

// strict L, strict U and D from A's CSR (the common tail of split and
// create_L_and_split)
void split_parts(mmatrix* A, mmatrix* L, mmatrix* U, mmatrix* D) {
  const int n = A->n;
  int nl = 0, nu = 0;
  for (int i = 0; i < n; ++i)
    for (int k = A->csr_ia[i]; k < A->csr_ia[i + 1]; ++k) {
      nl += A->csr_ja[k] < i;
      nu += A->csr_ja[k] > i;
    }
  alloc_csr(L, n, nl);
  alloc_csr(U, n, nu);
  alloc_csr(D, n, n);
  int il = 0, iu = 0;
  for (int i = 0; i < n; ++i) {
    L->csr_ia[i] = il;
    U->csr_ia[i] = iu;
    for (int k = A->csr_ia[i]; k < A->csr_ia[i + 1]; ++k) {
      const int c = A->csr_ja[k];
      if (c == i) {
        D->csr_vals[i] = A->csr_vals[k];
        D->csr_ia[i] = i;
        D->csr_ja[i] = i;
      } else if (c < i) {
        L->csr_ja[il] = c;
        L->csr_vals[il++] = A->csr_vals[k];
      } else {
        U->csr_ja[iu] = c;
        U->csr_vals[iu++] = A->csr_vals[k];
      }
    }
  }
  L->csr_ia[n] = il;
  U->csr_ia[n] = iu;
  D->csr_ia[n] = n;
  L->n = U->n = D->n = n;
  L->m = U->m = D->m = A->m;
  L->nnz = L->nnz_unpacked = il;
  U->nnz = U->nnz_unpacked = iu;
  D->nnz = D->nnz_unpacked = n;
}
}  // namespace

// io_utils.c:268-363
extern "C" void split(mmatrix* A, mmatrix* L, mmatrix* U, mmatrix* D) { split_parts(A, L, U, D); }

// io_utils.c:367-491: adjacency (with unit diagonal placeholders) -> graph
// Laplacian in place, then split.  Degrees are summed into an int exactly as
// the reference does (io_utils.c:387-395), so non-integer edge weights are
// truncated; weighted=1 builds the normalised Laplacian with unit diagonal.
extern "C" void create_L_and_split(mmatrix* A, mmatrix* L, mmatrix* U, mmatrix* D, int weighted) {
  const int n = A->n;
  std::vector<int> deg(n, 0);
  for (int i = 0; i < n; ++i) {
    int d = -1;
    for (int k = A->csr_ia[i]; k < A->csr_ia[i + 1]; ++k) d += A->csr_vals[k];  // int accumulation
    deg[i] = d;
  }
  for (int i = 0; i < n; ++i) {
    const double dsq = weighted ? 1.0 / sqrt((double)deg[i]) : 0.0;
    for (int k = A->csr_ia[i]; k < A->csr_ia[i + 1]; ++k) {
      const int c = A->csr_ja[k];
      if (c == i) A->csr_vals[k] = weighted ? 1.0 : (double)deg[i];
      else if (!weighted) A->csr_vals[k] = -A->csr_vals[k];
      else A->csr_vals[k] = (-1.0) * A->csr_vals[k] * dsq * (1.0 / sqrt((double)deg[c]));
    }
  }
  split_parts(A, L, U, D);
}
