// noalloc.cu -- gb_dot_noalloc: a dot product that allocates no device memory.
//
// cuda_dot (lap_abi.cu) keeps its block partials, completion ticket and
// result slot in device buffers that it cudaMallocs on its first call.  Some
// callers cannot let a library allocate:
//   * processes whose device memory is already claimed by another allocator
//     (a framework's caching allocator that reserved the GPU up front), where
//     a late cudaMalloc fails with out-of-memory;
//   * latency-critical loops that keep work in flight on other streams, where
//     the implicit synchronisation cudaMalloc / cudaFree may perform would
//     stall that work.
// This variant keeps the same three pieces of scratch in one file-scope
// __device__ array, created with the module, so a call only launches
// kernels and copies the 8-byte result back.
//
// Limits and rules of use:
//   * one partial per 4096-element chunk, kNoallocSlots partials: n is at
//     most GB_DOT_NOALLOC_MAX_N; a larger n is rejected with GB_BAD_INPUT and
//     a message on stderr, before any device work;
//   * the first call on each device (that device current) looks the array's
//     address up with cudaGetSymbolAddress -- setup that may load the module
//     -- so make the first call before any stream capture begins;
//   * there is one scratch array per device and process: calls that can
//     overlap on a device (several host threads, or unordered streams) race
//     on it and return wrong sums.  Serialise them;
//   * every call blocks the calling thread: it copies the 8-byte result into
//     the caller's host variable and waits for the stream;
//   * the completion ticket must be zero when the kernel starts: every call
//     clears it on its stream before the launch, and the last block clears it
//     again on the way out.  Partials and the result slot are written before
//     they are read and need no clearing.
// The chunking is fixed, so the sum's rounding depends on n only, not on the
// GPU's SM count; it may differ from cuda_dot's in the last bits.
#include <algorithm>
#include <atomic>
#include <cstdio>

#include "gb_common.cuh"
#include "gblap.h"
#include "kernels.h"

using namespace gb;

namespace {

constexpr int kNoallocChunk = 4096;  // elements per partial
constexpr int kNoallocSlots = GB_DOT_NOALLOC_MAX_N / kNoallocChunk;
static_assert((long long)kNoallocSlots * kNoallocChunk == GB_DOT_NOALLOC_MAX_N, "limit layout");

// [0, 256): ticket (unsigned) at 0, result (double) at 8; then the partials.
constexpr int kNoallocHeader = 256;
constexpr int kNoallocBytes = kNoallocHeader + kNoallocSlots * (int)sizeof(double);

static __device__ __align__(256) unsigned char g_dot_noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
std::atomic<unsigned char*> g_scratch_addr[kMaxDevices];

__global__ void __launch_bounds__(kRedThreads)
    dot_noalloc_kernel(int n, const double* __restrict__ v, const double* __restrict__ w,
                       unsigned char* scratch) {
  unsigned* ticket = reinterpret_cast<unsigned*>(scratch);
  double* out = reinterpret_cast<double*>(scratch + 8);
  double* part = reinterpret_cast<double*>(scratch + kNoallocHeader);
  __shared__ double sm[kRedThreads / 32];
  __shared__ bool last;
  const int nchunks = (n + kNoallocChunk - 1) / kNoallocChunk;
  for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int i0 = c * kNoallocChunk;
    const int i1 = min(n, i0 + kNoallocChunk);
    double acc[1] = {0.0};
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) acc[0] = fma(v[i], w[i], acc[0]);
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) part[c] = acc[0];
    __syncthreads();  // sm is reused by the next chunk's sum
  }
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1u;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();  // acquire side: the other blocks' partials, read by every thread below
  // the last block: partials in chunk order, fixed per-thread striding
  double t[1] = {0.0};
  for (int c = threadIdx.x; c < nchunks; c += blockDim.x) t[0] += ld_relaxed(part + c);
  block_sum<1>(t, sm);
  if (threadIdx.x == 0) {
    *out = t[0];
    *ticket = 0u;
  }
}

// Address of this device's scratch array; looked up once per device.
int scratch_for_current_device(unsigned char** out) {
  int dev = -1;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return GB_NOT_SUPPORTED;
  unsigned char* p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    void* addr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_dot_noalloc_scratch);
    if (e != cudaSuccess || addr == nullptr) {
      std::fprintf(stderr, "gb_dot_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
                   cudaGetErrorString(e));
      return GB_CUDA_ERROR;
    }
    p = static_cast<unsigned char*>(addr);
    g_scratch_addr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return GB_OK;
}

}  // namespace

extern "C" int gb_dot_noalloc(int n, const double* v, const double* w, double* result_host,
                              void* stream) {
  if (result_host == nullptr || n < 0 || (n > 0 && (v == nullptr || w == nullptr))) return GB_BAD_INPUT;
  if (n > GB_DOT_NOALLOC_MAX_N) {
    std::fprintf(stderr,
                 "gb_dot_noalloc: n = %d exceeds the static scratch limit of %d elements "
                 "(use cuda_dot for longer vectors)\n",
                 n, GB_DOT_NOALLOC_MAX_N);
    return GB_BAD_INPUT;
  }
  unsigned char* scratch = nullptr;
  GB_TRY(scratch_for_current_device(&scratch));
  if (n == 0) {
    *result_host = 0.0;
    return GB_OK;
  }
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nchunks = (n + kNoallocChunk - 1) / kNoallocChunk;
  const int grid = std::max(1, std::min(nchunks, reduction_grid()));
  GB_CUDA_TRY(cudaMemsetAsync(scratch, 0, sizeof(unsigned), s));
  dot_noalloc_kernel<<<grid, kRedThreads, 0, s>>>(n, v, w, scratch);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaMemcpyAsync(result_host, scratch + 8, sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}
