// kernels.h -- host-side launchers of the generic kernels (kernels.cu).
#pragma once

#include "gblap_internal.h"

namespace gb {

int device_sm_count();
// Resident blocks per SM of `kernel` at this block size (cached); grids of
// the grid-stride kernels are sized to one full wave: SMs x this.
int occupancy_blocks(const void* kernel, int threads, size_t dyn_smem = 0);
template <typename K>
inline int wave_grid(K kernel, int threads, long long work_blocks) {
  const long long cap = (long long)device_sm_count() * occupancy_blocks((const void*)kernel, threads);
  return (int)(work_blocks < 1 ? 1 : (work_blocks < cap ? work_blocks : cap));
}

// Greedy row bundles for `rows_per_bundle` <= 32 rows and <= kBundleNnz entries.
int spmv_plan_build(int n, int nnz, const int* ia_host, SpmvPlan* plan, int rows_per_bundle);
void spmv_plan_free(SpmvPlan* plan);

// y = alpha*A*x + beta*y; plan may be null (plan-free 32-row bundles).
template <typename T>
int spmv_axpby(const SpmvPlan* plan, int n, const int* ia, const int* ja, const T* a, T alpha,
               const T* x, T beta, T* y, cudaStream_t s);

// Deterministic dot product; result written to *out_dev (device) and, if
// out_host != null, copied back (synchronises the stream).
int dot_dev(int n, const double* v, const double* w, double* out_dev, double* part,
            unsigned* ticket, cudaStream_t s);

int axpy_dev(int n, double alpha, const double* x, double* y, cudaStream_t s);
int scal_dev(int n, double alpha, double* v, cudaStream_t s);
int vec_vec_dev(int n, const double* x, const double* y, double* res, cudaStream_t s);
int reciprocal_dev(int n, const double* v, double* res, cudaStream_t s);
int sqrt_dev(int n, const double* v, double* res, cudaStream_t s);
int copy_dev(int n, const double* src, double* dst, cudaStream_t s);
int fill_dev(int n, double v, double* dst, cudaStream_t s);
int fill_sentinel_dev(int n, double* dst, cudaStream_t s);
int fill_sentinel_dev(int n, float* dst, cudaStream_t s);
int cast_f64_to_f32(int n, const double* src, float* dst, cudaStream_t s);
int cast_f32_to_f64(int n, const float* src, double* dst, cudaStream_t s);
int gather_values(int n, const int* map, const double* src, double* dst, float* dst32,
                  cudaStream_t s);

int reduction_grid();

// Fingerprint of a CSR pattern (ia [n+1], ja [nnz]): the sum modulo 2^64 of
// a 64-bit mix of every (array, position, value), so it does not depend on
// summation order and the device and host versions agree.  Caches keyed by
// array addresses compare it on every call, so new contents behind an old
// address are noticed.
__host__ __device__ inline unsigned long long pattern_mix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ inline unsigned long long pattern_elem(unsigned long long array, long long pos, int v) {
  return pattern_mix(pattern_mix(array * 0xD6E8FEB86659FD93ull + (unsigned long long)pos) ^ (unsigned)v);
}
unsigned long long pattern_hash_host(int n, int nnz, const int* ia, const int* ja);
// Device arrays; dev_out is 8 bytes of device scratch.  Synchronises s.
int pattern_hash(int n, int nnz, const int* ia, const int* ja, unsigned long long* dev_out, cudaStream_t s,
                 unsigned long long* out);

}  // namespace gb
