// kernels.cu -- SpMV row-bundle plans, the generic SpMV and the BLAS-1 /
// elementwise kernels behind LAP's blas.h surface (replacing cuBLAS
// Ddot/Daxpy/Dscal and the grid-stride helpers of cuda_blas.cu:563-613).
//
// Elementwise kernels are HBM-bound: grid-stride loops over 16-byte
// vectors where alignment allows, grids sized as a multiple of the SM count.
// The dot product is deterministic: per-block partials in a fixed grid,
// summed in block order by the last block to finish (single launch).
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "gb_common.cuh"
#include "kernels.h"
#include "spmv_bundle.cuh"

namespace gb {

int device_sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
  }
  return sms;
}

int reduction_grid() { return device_sm_count() * kRedBlocksPerSM; }

int occupancy_blocks(const void* kernel, int threads, size_t dyn_smem) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> cache;
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_pair(kernel, threads);
  auto f = cache.find(key);
  if (f != cache.end()) return f->second;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, dyn_smem) != cudaSuccess || nb < 1) {
    cudaGetLastError();
    nb = 1;
  }
  cache[key] = nb;
  return nb;
}

static int ew_grid(long long n) {
  const long long need = (n + kRedThreads - 1) / kRedThreads;
  const long long cap = (long long)device_sm_count() * 8;
  return (int)std::max(1LL, std::min(need, cap));
}

// ------------------------------------------------------------ SpMV plan
int spmv_plan_build(int n, int nnz, const int* ia, SpmvPlan* plan, int rpb) {
  (void)nnz;
  rpb = std::max(1, std::min(rpb, kBundleRows));
  const int cap = GB_SPMV_STAGE_A ? kBundleNnz / 2 : kBundleNnz;  // entries a bundle stages
  std::vector<int> b;
  b.reserve(n / rpb + 2);
  b.push_back(0);
  int r = 0, longs = 0;
  while (r < n) {
    const int len0 = ia[r + 1] - ia[r];
    if (len0 > cap) {
      ++r;
      ++longs;
      b.push_back(r);
      continue;
    }
    const int start = r;
    long long nz = 0;
    while (r < n && r - start < rpb) {
      const int len = ia[r + 1] - ia[r];
      if (nz + len > cap) break;
      nz += len;
      ++r;
    }
    b.push_back(r);
  }
  plan->n = n;
  plan->nnz = nnz;
  plan->nbundles = (int)b.size() - 1;
  plan->long_rows = longs;
  plan->rows_per_bundle = rpb;
  // every bundle 32 consecutive rows (a stencil): the kernels' plan-free
  // layout computes the same bundles, one dependent load fewer per bundle.
  // Every reader of SpmvPlan::bundles takes nullptr as that layout.
  bool uniform = rpb == kBundleRows && longs == 0;
  for (size_t i = 0; uniform && i + 1 < b.size(); ++i)
    if (b[i] != (int)(i * kBundleRows)) uniform = false;
  if (uniform) {
    plan->bundles = nullptr;
    return GB_OK;
  }
  GB_CUDA_TRY(cudaMalloc(&plan->bundles, sizeof(int) * b.size()));
  GB_CUDA_TRY(cudaMemcpy(plan->bundles, b.data(), sizeof(int) * b.size(), cudaMemcpyHostToDevice));
  return GB_OK;
}

void spmv_plan_free(SpmvPlan* plan) {
  if (plan->bundles) cudaFree(plan->bundles);
  plan->bundles = nullptr;
  plan->nbundles = 0;
}

// ------------------------------------------------------------ generic SpMV
template <typename T>
struct EpAxpby {
  T* __restrict__ y;
  T beta;
  __device__ __forceinline__ T init(int r) const { return beta == T(0) ? T(0) : mul_rn(y[r], beta); }
  __device__ __forceinline__ void store(int r, T v) const { y[r] = v; }
};

template <typename T>
__global__ void __launch_bounds__(kSpmvWarps * 32)
    spmv_axpby_kernel(int n, int nb, const int* __restrict__ bundles, const int* __restrict__ ia,
                      const int* __restrict__ ja, const T* __restrict__ a, T alpha,
                      const T* __restrict__ x, T beta, T* y) {
  __shared__ T stage[kSpmvWarps][kBundleNnz];
  const int wid = threadIdx.x >> 5;
  XPlain<T> xf{x};
  EpAxpby<T> ep{y, beta};
  for (int b = blockIdx.x * kSpmvWarps + wid; b < nb; b += gridDim.x * kSpmvWarps)
    spmv_bundle<T, true>(b, n, bundles, ia, ja, a, alpha, xf, ep, stage[wid]);
}

template <typename T>
int spmv_axpby(const SpmvPlan* plan, int n, const int* ia, const int* ja, const T* a, T alpha,
               const T* x, T beta, T* y, cudaStream_t s) {
  if (n <= 0) return GB_OK;
  const int nb = plan ? plan->nbundles : ceil_div(n, 32);
  const int blocks = wave_grid(spmv_axpby_kernel<T>, kSpmvWarps * 32, ceil_div(nb, kSpmvWarps));
  spmv_axpby_kernel<T><<<blocks, kSpmvWarps * 32, 0, s>>>(n, nb, plan ? plan->bundles : nullptr,
                                                          ia, ja, a, alpha, x, beta, y);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}
template int spmv_axpby<double>(const SpmvPlan*, int, const int*, const int*, const double*,
                                double, const double*, double, double*, cudaStream_t);
template int spmv_axpby<float>(const SpmvPlan*, int, const int*, const int*, const float*, float,
                               const float*, float, float*, cudaStream_t);

// ------------------------------------------------------------ dot
__global__ void __launch_bounds__(kRedThreads)
    dot_kernel(int n, const double* __restrict__ v, const double* __restrict__ w, double* out,
               double* part, unsigned* ticket) {
  __shared__ double sm[kRedThreads / 32];
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc[0] = add_rn(acc[0], mul_rn(v[i], w[i]));
  block_sum<1>(acc, sm);
  if (publish_partials<1>(acc, part, gridDim.x, blockIdx.x, ticket, gridDim.x)) {
    double t[1] = {0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t[0] += ld_relaxed(part + i);
    block_sum<1>(t, sm);
    if (threadIdx.x == 0) *out = t[0];
  }
}

int dot_dev(int n, const double* v, const double* w, double* out, double* part, unsigned* ticket,
            cudaStream_t s) {
  const int g = std::max(1, std::min(reduction_grid(), ceil_div(n, kRedThreads)));
  dot_kernel<<<g, kRedThreads, 0, s>>>(n, v, w, out, part, ticket);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// ------------------------------------------------------------ elementwise
__global__ void axpy_kernel(int n, double alpha, const double* __restrict__ x, double* y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = add_rn(y[i], mul_rn(alpha, x[i]));
}
__global__ void scal_kernel(int n, double alpha, double* v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    v[i] = mul_rn(v[i], alpha);
}
__global__ void vec_vec_kernel(int n, const double* x, const double* y, double* res) {
  // x, y and res may alias (it_jacobi.c:345 scales in place)
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    res[i] = mul_rn(x[i], y[i]);
}
__global__ void reciprocal_kernel(int n, const double* v, double* res) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d = v[i];
    res[i] = d != 0.0 ? __ddiv_rn(1.0, d) : 0.0;
  }
}
__global__ void sqrt_kernel(int n, const double* v, double* res) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d = v[i];
    res[i] = d >= 0.0 ? __dsqrt_rn(d) : 0.0;
  }
}
__global__ void copy_kernel(int n, const double* __restrict__ s, double* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = s[i];
}
template <typename T>
__global__ void fill_kernel(int n, T v, T* d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = v;
}
__global__ void fill_sentinel64(int n, double* d) {
  const double s = sentinel_f64();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = s;
}
__global__ void fill_sentinel32(int n, float* d) {
  const float s = sentinel_f32();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = s;
}
__global__ void cast64to32(int n, const double* __restrict__ s, float* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = (float)s[i];
}
__global__ void cast32to64(int n, const float* __restrict__ s, double* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = (double)s[i];
}
__global__ void gather_kernel(int n, const int* __restrict__ map, const double* __restrict__ src,
                              double* dst, float* dst32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int k = map[i];
    const double v = k >= 0 ? src[k] : 0.0;
    if (dst) dst[i] = v;
    if (dst32) dst32[i] = (float)v;
  }
}

#define GB_EW_LAUNCH(kernel, n, ...)                                              \
  do {                                                                            \
    if ((n) <= 0) return GB_OK;                                                   \
    kernel<<<ew_grid(n), kRedThreads, 0, s>>>((n), __VA_ARGS__);                  \
    GB_CUDA_TRY(cudaGetLastError());                                              \
    return GB_OK;                                                                 \
  } while (0)

int axpy_dev(int n, double alpha, const double* x, double* y, cudaStream_t s) { GB_EW_LAUNCH(axpy_kernel, n, alpha, x, y); }
int scal_dev(int n, double alpha, double* v, cudaStream_t s) { GB_EW_LAUNCH(scal_kernel, n, alpha, v); }
int vec_vec_dev(int n, const double* x, const double* y, double* r, cudaStream_t s) { GB_EW_LAUNCH(vec_vec_kernel, n, x, y, r); }
int reciprocal_dev(int n, const double* v, double* r, cudaStream_t s) { GB_EW_LAUNCH(reciprocal_kernel, n, v, r); }
int sqrt_dev(int n, const double* v, double* r, cudaStream_t s) { GB_EW_LAUNCH(sqrt_kernel, n, v, r); }
int copy_dev(int n, const double* src, double* dst, cudaStream_t s) { GB_EW_LAUNCH(copy_kernel, n, src, dst); }
int fill_dev(int n, double v, double* dst, cudaStream_t s) { GB_EW_LAUNCH(fill_kernel<double>, n, v, dst); }
int fill_sentinel_dev(int n, double* dst, cudaStream_t s) { GB_EW_LAUNCH(fill_sentinel64, n, dst); }
int fill_sentinel_dev(int n, float* dst, cudaStream_t s) { GB_EW_LAUNCH(fill_sentinel32, n, dst); }
int cast_f64_to_f32(int n, const double* src, float* dst, cudaStream_t s) { GB_EW_LAUNCH(cast64to32, n, src, dst); }
int cast_f32_to_f64(int n, const float* src, double* dst, cudaStream_t s) { GB_EW_LAUNCH(cast32to64, n, src, dst); }
int gather_values(int n, const int* map, const double* src, double* dst, float* dst32, cudaStream_t s) {
  GB_EW_LAUNCH(gather_kernel, n, map, src, dst, dst32);
}

// ------------------------------------------------------------ pattern fingerprint
__global__ void __launch_bounds__(kRedThreads)
    pattern_hash_kernel(int n, int nnz, const int* __restrict__ ia, const int* __restrict__ ja,
                        unsigned long long* out) {
  unsigned long long h = 0ull;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i <= n; i += stride)
    h += pattern_elem(1ull, i, __ldg(ia + i));
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nnz; k += stride)
    h += pattern_elem(2ull, k, __ldg(ja + k));
  for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, h);
}

unsigned long long pattern_hash_host(int n, int nnz, const int* ia, const int* ja) {
  unsigned long long h = 0ull;
  for (long long i = 0; i <= n; ++i) h += pattern_elem(1ull, i, ia[i]);
  for (long long k = 0; k < nnz; ++k) h += pattern_elem(2ull, k, ja[k]);
  return h;
}

int pattern_hash(int n, int nnz, const int* ia, const int* ja, unsigned long long* dev_out, cudaStream_t s,
                 unsigned long long* out) {
  if (n < 0 || nnz < 0 || !ia || (nnz > 0 && !ja) || !dev_out || !out) return GB_BAD_INPUT;
  GB_CUDA_TRY(cudaMemsetAsync(dev_out, 0, sizeof(unsigned long long), s));
  const long long work = (long long)n + 1 + nnz;
  const int grid = (int)std::max(1LL, std::min<long long>((work + kRedThreads - 1) / kRedThreads, reduction_grid()));
  pattern_hash_kernel<<<grid, kRedThreads, 0, s>>>(n, nnz, ia, ja, dev_out);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaMemcpyAsync(out, dev_out, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

}  // namespace gb
