// lap_abi.cu -- LAP's CUDA backend surface (cuda_blas.h, devMem.h) and the
// backend-neutral blas.h layer, implemented on libgblap's kernels.
//
// Same symbols, argument meaning and pointer conventions as cuda_blas.cu /
// devMem.cpp / blas.c built with -DCUDA=1, so LAP's own solver and driver
// sources link against this library unchanged.  Everything runs on the
// legacy default stream, as LAP's cuBLAS/cuSPARSE handles do, so it orders
// with the caller's cudaMemcpy calls; dot() returns a host scalar.
//
// State: LAP keeps global handles, buffers and one analysis per factor
// (cuda_blas.cu:10-25).  Here the analyses (level schedules) are cached per
// factor, keyed by its row-pointer address and sizes, so several matrices
// can be live at once; initialize_* functions build them eagerly and the
// solves build a missing one on first use.  Every use recomputes the
// pattern's fingerprint (pattern_hash, one pass over ia and ja) and rebuilds
// the analysis when it changed: a factor freed and reallocated at the same
// address with another pattern never runs a stale schedule.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "gb_common.cuh"
#include "kernels.h"
#include "lap_gblap.h"
#include "sptrsv.h"

using namespace gb;

namespace {

struct Scratch {
  unsigned long long* hash = nullptr;
  double* part = nullptr;
  unsigned* ticket = nullptr;
  double* out = nullptr;
  int* err = nullptr;
  double* tmp = nullptr;
  int tmp_len = 0;
  int part_len = 0;
};

struct TriEntry {
  TriPlan plan;
  unsigned long long hash = 0;
  ~TriEntry() { tri_plan_free(&plan); }
};

struct IcEntry {
  int n = 0, nnz = 0;
  unsigned long long hash = 0;
  TriPlan lower, upper;
  int* dpos = nullptr;
  int* tpos = nullptr;
  int* done = nullptr;
  unsigned* ticket = nullptr;
  int* zpiv = nullptr;
  ~IcEntry() {
    tri_plan_free(&lower);
    tri_plan_free(&upper);
    for (void* p : {(void*)dpos, (void*)tpos, (void*)done, (void*)ticket, (void*)zpiv})
      if (p) cudaFree(p);
  }
};

std::mutex g_mu;
Scratch g_s;
// heap-held and never destroyed: no cudaFree runs during static destruction
// at exit, after the CUDA runtime may have shut down
auto& g_tri = *new std::map<std::tuple<const void*, int, int, int>, std::unique_ptr<TriEntry>>;  // (ptr, n, nnz, lower)
auto& g_ic = *new std::map<std::tuple<const void*, int, int>, std::unique_ptr<IcEntry>>;

constexpr cudaStream_t kStream = 0;  // legacy default stream, as LAP's handles

int ensure_scratch() {
  if (g_s.part) return GB_OK;
  g_s.part_len = reduction_grid() + 8;
  GB_CUDA_TRY(cudaMalloc(&g_s.hash, sizeof(unsigned long long)));
  GB_CUDA_TRY(cudaMalloc(&g_s.part, sizeof(double) * g_s.part_len));
  GB_CUDA_TRY(cudaMalloc(&g_s.ticket, sizeof(unsigned) * 4));
  GB_CUDA_TRY(cudaMemset(g_s.ticket, 0, sizeof(unsigned) * 4));
  GB_CUDA_TRY(cudaMalloc(&g_s.out, sizeof(double) * 4));
  GB_CUDA_TRY(cudaMalloc(&g_s.err, sizeof(int) * 4));
  GB_CUDA_TRY(cudaMemset(g_s.err, 0, sizeof(int) * 4));
  return GB_OK;
}

int ensure_tmp(int n) {
  if (g_s.tmp_len >= n) return GB_OK;
  if (g_s.tmp) cudaFree(g_s.tmp);
  g_s.tmp = nullptr;
  GB_CUDA_TRY(cudaMalloc(&g_s.tmp, sizeof(double) * std::max(n, 1)));
  g_s.tmp_len = n;
  return GB_OK;
}

void report(const char* where, int rc) {
  if (rc != GB_OK) fprintf(stderr, "libgblap: %s: %s\n", where, gb_status_str(rc));
}

int copy_structure(int n, int nnz, const int* ia, const int* ja, std::vector<int>* hia,
                   std::vector<int>* hja) {
  hia->resize(n + 1);
  hja->resize(std::max(nnz, 1));
  GB_CUDA_TRY(cudaMemcpy(hia->data(), ia, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
  if (nnz > 0) GB_CUDA_TRY(cudaMemcpy(hja->data(), ja, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
  if ((*hia)[0] != 0 || (*hia)[n] > nnz) return GB_BAD_INPUT;
  return GB_OK;
}

// Level schedule of a factor with its diagonal embedded (LAP GPU convention).
int get_tri(int n, int nnz, const int* ia, const int* ja, bool lower, TriEntry** out) {
  auto key = std::make_tuple((const void*)ia, n, nnz, lower ? 1 : 0);
  unsigned long long h = 0;
  GB_TRY(pattern_hash(n, nnz, ia, ja, g_s.hash, kStream, &h));
  auto it = g_tri.find(key);
  if (it != g_tri.end()) {
    if (it->second->hash == h) {
      *out = it->second.get();
      return GB_OK;
    }
    g_tri.erase(it);  // new pattern behind the same address
  }
  std::vector<int> hia, hja;
  GB_TRY(copy_structure(n, nnz, ia, ja, &hia, &hja));
  TriDeps d;
  GB_TRY(deps_embedded(n, hia.data(), hja.data(), lower, &d));
  auto e = std::make_unique<TriEntry>();
  e->hash = h;
  GB_TRY(tri_plan_build(d, &e->plan));
  *out = e.get();
  g_tri[key] = std::move(e);
  return GB_OK;
}

int get_ic(int n, int nnz, const int* ia, const int* ja, IcEntry** out) {
  auto key = std::make_tuple((const void*)ia, n, nnz);
  unsigned long long h = 0;
  GB_TRY(pattern_hash(n, nnz, ia, ja, g_s.hash, kStream, &h));
  auto it = g_ic.find(key);
  if (it != g_ic.end()) {
    if (it->second->hash == h) {
      *out = it->second.get();
      return GB_OK;
    }
    g_ic.erase(it);  // new pattern behind the same address
  }
  std::vector<int> hia, hja, tpos, dpos(n, -1);
  GB_TRY(copy_structure(n, nnz, ia, ja, &hia, &hja));
  for (int i = 0; i < n; ++i)
    for (int k = hia[i]; k < hia[i + 1]; ++k)
      if (hja[k] == i) dpos[i] = k;
  for (int i = 0; i < n; ++i)
    if (dpos[i] < 0) return GB_BAD_INPUT;
  GB_TRY(transpose_positions(n, hia.data(), hja.data(), &tpos));
  TriDeps dl, du;
  GB_TRY(deps_ichol(n, hia.data(), hja.data(), tpos, true, &dl));
  GB_TRY(deps_ichol(n, hia.data(), hja.data(), tpos, false, &du));
  auto e = std::make_unique<IcEntry>();
  e->n = n;
  e->nnz = nnz;
  e->hash = h;
  GB_TRY(tri_plan_build(dl, &e->lower));
  GB_TRY(tri_plan_build(du, &e->upper));
  GB_CUDA_TRY(cudaMalloc(&e->dpos, sizeof(int) * n));
  GB_CUDA_TRY(cudaMemcpy(e->dpos, dpos.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  GB_CUDA_TRY(cudaMalloc(&e->tpos, sizeof(int) * std::max(nnz, 1)));
  GB_CUDA_TRY(cudaMemcpy(e->tpos, tpos.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice));
  GB_CUDA_TRY(cudaMalloc(&e->done, sizeof(int) * n));
  GB_CUDA_TRY(cudaMalloc(&e->ticket, sizeof(unsigned) * 4));
  GB_CUDA_TRY(cudaMemset(e->ticket, 0, sizeof(unsigned) * 4));
  GB_CUDA_TRY(cudaMalloc(&e->zpiv, sizeof(int)));
  *out = e.get();
  g_ic[key] = std::move(e);
  return GB_OK;
}

int check_err(const char* where) {
  int err = 0;
  if (cudaMemcpy(&err, g_s.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return GB_CUDA_ERROR;
  if (err) {
    fprintf(stderr, "libgblap: %s: %s\n", where, gb_status_str(err));
    cudaMemset(g_s.err, 0, sizeof(int));
  }
  return err;
}

__global__ void copy_lower_kernel(int n, const int* __restrict__ ia, const int* __restrict__ dpos,
                                  const double* __restrict__ f, double* a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = ia[i]; k <= dpos[i]; ++k) a[k] = f[k];
}

}  // namespace

// ============================================================ cuda_blas.h
extern "C" double cuda_dot(const int n, const double* v, const double* w) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (ensure_scratch() != GB_OK) return 0.0;
  int rc = dot_dev(n, v, w, g_s.out, g_s.part, g_s.ticket, kStream);
  double r = 0.0;
  if (n <= 0) return 0.0;
  if (rc == GB_OK && cudaMemcpy(&r, g_s.out, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = GB_CUDA_ERROR;
  report("cuda_dot", rc);
  return r;
}

extern "C" void cuda_scal(const int n, const double alpha, double* v) { report("cuda_scal", scal_dev(n, alpha, v, kStream)); }
extern "C" void cuda_axpy(const int n, const double alpha, const double* x, double* y) { report("cuda_axpy", axpy_dev(n, alpha, x, y, kStream)); }
extern "C" void cuda_vec_vec(const int n, const double* x, const double* y, double* res) { report("cuda_vec_vec", vec_vec_dev(n, x, y, res, kStream)); }
extern "C" void cuda_vector_sqrt(const int n, const double* v, double* res) { report("cuda_vector_sqrt", sqrt_dev(n, v, res, kStream)); }
extern "C" void cuda_vector_reciprocal(const int n, const double* v, double* res) { report("cuda_vector_reciprocal", reciprocal_dev(n, v, res, kStream)); }
extern "C" void cuda_vec_copy(const int n, const double* src, double* dest) { report("cuda_vec_copy", copy_dev(n, src, dest, kStream)); }
extern "C" void cuda_vec_zero(const int n, double* vec) { report("cuda_vec_zero", fill_dev(n, 0.0, vec, kStream)); }

extern "C" void cuda_csr_matvec(const int n, const int nnz, const int* ia, const int* ja,
                                const double* a, const double* x, double* result,
                                const double* al, const double* bet) {
  (void)nnz;
  report("cuda_csr_matvec", spmv_axpby<double>(nullptr, n, ia, ja, a, *al, x, *bet, result, kStream));
}

static void tri_solve_embedded(const char* where, bool lower, int n, int nnz, const int* p,
                               const int* j, const double* v, const double* x, double* y) {
  std::lock_guard<std::mutex> lk(g_mu);
  int rc = ensure_scratch();
  TriEntry* e = nullptr;
  if (rc == GB_OK) rc = get_tri(n, nnz, p, j, lower, &e);
  if (rc == GB_OK) rc = tri_plan_fill(&e->plan, v, v, kFillExact, kStream);
  if (rc == GB_OK) rc = tri_solve_plain(&e->plan, x, y, g_s.err, kStream);
  report(where, rc);
}

extern "C" void cuda_lower_triangular_solve(const int n, const int nnz, const int* lia,
                                            const int* lja, const double* la, const double* diag,
                                            const double* x, double* result) {
  (void)diag;  // LAP's GPU solves take the diagonal from inside L (cuda_blas.cu:731-776)
  tri_solve_embedded("cuda_lower_triangular_solve", true, n, nnz, lia, lja, la, x, result);
}

extern "C" void cuda_upper_triangular_solve(const int n, const int nnz, const int* uia,
                                            const int* uja, const double* ua, const double* diag,
                                            const double* x, double* result) {
  (void)diag;
  tri_solve_embedded("cuda_upper_triangular_solve", false, n, nnz, uia, uja, ua, x, result);
}

extern "C" void initialize_handles(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  report("initialize_handles", ensure_scratch());
}

extern "C" void initialize_spmv_buffer(const int n, const int nnz, int* ia, int* ja, double* a,
                                       const double* x, double* result, double* al, double* bet) {
  // the row-bundle SpMV needs no per-matrix buffer (cuda_blas.cu:34-97 sizes one)
  (void)n; (void)nnz; (void)ia; (void)ja; (void)a; (void)x; (void)result; (void)al; (void)bet;
  initialize_handles();
}

extern "C" void initialize_and_analyze_L_and_U_solve(const int n, const int nnzL, int* lia,
                                                     int* lja, double* la, const int nnzU,
                                                     int* uia, int* uja, double* ua) {
  (void)la; (void)ua;
  std::lock_guard<std::mutex> lk(g_mu);
  TriEntry* e = nullptr;
  int rc = ensure_scratch();
  if (rc == GB_OK) rc = get_tri(n, nnzL, lia, lja, true, &e);
  if (rc == GB_OK) rc = get_tri(n, nnzU, uia, uja, false, &e);
  report("initialize_and_analyze_L_and_U_solve", rc);
}

extern "C" void initialize_L_and_U_descriptors(const int n, const int nnzL, int* lia, int* lja,
                                               double* la, const int nnzU, int* uia, int* uja,
                                               double* ua) {
  (void)n; (void)nnzL; (void)lia; (void)lja; (void)la; (void)nnzU; (void)uia; (void)uja; (void)ua;
}

// IC(0) in place on A's full pattern: the lower triangle (diagonal included)
// receives L, the upper triangle is left as it was -- cusparseDcsric02's
// contract (cuda_blas.cu:261-488).  A zero/negative pivot is reported on
// stderr, as the reference's zero-pivot query does.
extern "C" void initialize_ichol(const int n, const int nnzA, int* ia, int* ja, double* a) {
  std::lock_guard<std::mutex> lk(g_mu);
  IcEntry* e = nullptr;
  int rc = ensure_scratch();
  if (rc == GB_OK) rc = get_ic(n, nnzA, ia, ja, &e);
  double* f = nullptr;
  if (rc == GB_OK && cudaMalloc(&f, sizeof(double) * std::max(nnzA, 1)) != cudaSuccess) rc = GB_NO_MEMORY;
  if (rc == GB_OK)
    rc = ichol_factor_dev(n, ia, ja, a, e->dpos, e->tpos, &e->lower, f, e->done, e->ticket, e->zpiv,
                          g_s.err, kStream);
  if (rc == GB_OK) {
    copy_lower_kernel<<<std::max(1, std::min(device_sm_count() * 8, ceil_div(n, 256))), 256>>>(
        n, ia, e->dpos, f, a);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = GB_CUDA_ERROR;
  }
  if (f) cudaFree(f);
  if (rc == GB_OK) {
    int zp = 0;
    cudaMemcpy(&zp, e->zpiv, sizeof(int), cudaMemcpyDeviceToHost);
    if (zp) fprintf(stderr, "libgblap: initialize_ichol: L(%d,%d) is not positive\n", zp - 1, zp - 1);
    rc = check_err("initialize_ichol");
  }
  report("initialize_ichol", rc);
}

// y = (L L^T)^{-1} x with L in the lower triangle of prec_data->ichol_vals on
// A's pattern; aux_vec1 holds L^{-1} x (cuda_blas.cu:490-561).
extern "C" void cuda_ichol(const int* ia, const int* ja, double* a, const int nnzA,
                           pdata* prec_data, double* x, double* y) {
  (void)a;
  std::lock_guard<std::mutex> lk(g_mu);
  IcEntry* e = nullptr;
  const int n = prec_data->n;
  int rc = ensure_scratch();
  if (rc == GB_OK) rc = get_ic(n, nnzA, ia, ja, &e);
  if (rc == GB_OK) rc = tri_plan_fill(&e->lower, prec_data->ichol_vals, prec_data->ichol_vals, kFillExact, kStream);
  if (rc == GB_OK) rc = tri_plan_fill(&e->upper, prec_data->ichol_vals, prec_data->ichol_vals, kFillExact, kStream);
  if (rc == GB_OK) rc = tri_solve_plain(&e->lower, x, prec_data->aux_vec1, g_s.err, kStream);
  if (rc == GB_OK) rc = tri_solve_plain(&e->upper, prec_data->aux_vec1, y, g_s.err, kStream);
  report("cuda_ichol", rc);
}

// ============================================================ devMem.h
extern "C" void* mallocForDevice(void* x, int n, int size) {
  (void)x;
  void* p = nullptr;
  const cudaError_t e = cudaMalloc(&p, (size_t)n * (size_t)size);
  if (e != cudaSuccess) {
    fprintf(stderr, "libgblap: mallocForDevice(%d x %d bytes): %s\n", n, size, cudaGetErrorString(e));
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

extern "C" void memcpyDevice(void* dest, void* src, int n, int size, char* type) {
  cudaMemcpyKind kind;
  if (strcmp(type, "H2D") == 0) kind = cudaMemcpyHostToDevice;
  else if (strcmp(type, "D2H") == 0) kind = cudaMemcpyDeviceToHost;
  else if (strcmp(type, "D2D") == 0) kind = cudaMemcpyDeviceToDevice;  // devMem.cpp:33-35 used D2H
  else {
    fprintf(stderr, "libgblap: memcpyDevice: unknown direction '%s'\n", type);
    return;
  }
  const cudaError_t e = cudaMemcpy(dest, src, (size_t)n * (size_t)size, kind);
  if (e != cudaSuccess) fprintf(stderr, "libgblap: memcpyDevice(%s): %s\n", type, cudaGetErrorString(e));
}

extern "C" void freeDevice(void* p) { cudaFree(p); }

// ============================================================ blas.h
extern "C" double dot(const int n, const double* v, const double* w) { return cuda_dot(n, v, w); }
extern "C" void axpy(const int n, const double alpha, double* x, double* y) { cuda_axpy(n, alpha, x, y); }
extern "C" void scal(const int n, const double alpha, double* v) { cuda_scal(n, alpha, v); }
extern "C" void csr_matvec(const int n, const int nnz, const int* ia, const int* ja, const double* a,
                           const double* x, double* result, const double* al, const double* bet,
                           const char* kind) {
  (void)kind;
  cuda_csr_matvec(n, nnz, ia, ja, a, x, result, al, bet);
}
extern "C" void lower_triangular_solve(const int n, const int nnz, const int* lia, const int* lja,
                                       const double* la, const double* diag, const double* x,
                                       double* result) {
  cuda_lower_triangular_solve(n, nnz, lia, lja, la, diag, x, result);
}
extern "C" void upper_triangular_solve(const int n, const int nnz, const int* uia, const int* uja,
                                       const double* ua, const double* diag, const double* x,
                                       double* result) {
  cuda_upper_triangular_solve(n, nnz, uia, uja, ua, diag, x, result);
}
extern "C" void ichol(const int* ia, const int* ja, double* a, const int nnzA, pdata* prec_data,
                      double* x, double* y) {
  cuda_ichol(ia, ja, a, nnzA, prec_data, x, y);
}
extern "C" void vec_vec(const int n, const double* x, double* y, double* res) { cuda_vec_vec(n, x, y, res); }
extern "C" void vector_reciprocal(const int n, const double* v, double* res) { cuda_vector_reciprocal(n, v, res); }
extern "C" void vector_sqrt(const int n, const double* v, double* res) { cuda_vector_sqrt(n, v, res); }
extern "C" void vec_copy(const int n, double* src, double* dest) { cuda_vec_copy(n, src, dest); }
extern "C" void vec_zero(const int n, double* vec) { cuda_vec_zero(n, vec); }
