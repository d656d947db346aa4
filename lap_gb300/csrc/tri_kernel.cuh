// tri_kernel.cuh -- tiled sync-free sparse triangular solve, TMA-staged.
//
// Replaces cusparseDcsrsv2_solve (cuda_blas.cu:731-820, :500, :516).  Every
// row is solved as simple_lower/upper_triangular_solve (simple_blas.c:46-85)
// does: acc = rhs; acc -= l_ij * y_j in the row's column order; y_i = acc /
// d_i.  EXACT keeps that rounding (separate mul and sub, a true division);
// otherwise the row uses FMAs and the precomputed reciprocal of d_i -- GB300
// runs FP64 at 1/64 of its FP32 rate, so every FP64 instruction on the
// dependency chain counts.
//
// Schedule (TriPlan, built on the host): rows are cut into contiguous tiles;
// inside a tile rows are grouped by their level with respect to the tile's
// own rows; each level is stored as one or more contiguous, 16-byte aligned
// RECORDS (rows, diagonal, reciprocal, dependency columns and values,
// column-major).  One CTA solves one tile at a time:
//   A) rhs of every row into shared memory (coalesced, tile-wide);
//   B) a producer warp streams the tile's records into a ring of shared
//      memory slots with cp.async.bulk (TMA), signalling an mbarrier per
//      slot; four consumer warps take the records in order: a dependency
//      inside the tile is read from shared memory (written at an earlier
//      level, ordered by a named barrier between levels), one in an earlier
//      tile from global memory by spinning on the producer's value (outputs
//      are pre-filled with a sentinel); results go to shared memory and
//      global memory;
//   C) per-row epilogue (fused vector updates, dot partials), coalesced.
// Tiles are taken by ticket in dependency order by a persistent grid, so a
// tile only waits on tiles already being solved by running CTAs.  Every
// wait (mbarrier or value) is bounded in wall-clock time; on expiry the
// error word is set and the CTA drains its own copies before leaving.
//
// OP contract:
//   void begin();  bool active();  void inactive_end()   (block 0, !active)
//   T rhs(int row);                 phase A
//   void done(int row, T y);        phase C
//   void chunk_end(tile_ix, ntiles, ticket, sm)   whole block, after the
//        tile; ticket[1] counts finished tiles (chunk_finished()).
#pragma once

#include "gb_common.cuh"
#include "kernels.h"
#include "spmv_bundle.cuh"

namespace gb {

constexpr int kTriConsumers = 4;                       // consumer warps
constexpr int kTriThreads = (kTriConsumers + 1) * 32;  // + one producer warp
constexpr int kTriSlots = 16;                          // ring depth (records in flight)
constexpr int kTriSlotBytes = 4096;                    // max record size
constexpr int kTriRecTable = 1024;                     // records of a tile cached in smem
constexpr int kRecLong = 2;                            // record flag: one row, warp-reduced
constexpr int kRecBarrier = 1;                         // record flag: level ends here

// Record header (16 bytes).  Layout after it, R4 = nrows rounded up to 4:
//   int rows[R4]; T diag[R4]; T dinv[R4]; int cols[len*R4]; T vals[len*R4]
// (LONG records: no cols/vals; they live at long_col/long_val[off ...]).
struct RecHdr {
  int nrows, len, flags, off;
};

template <typename T>
struct TriArgs {
  int ntiles;
  const int* __restrict__ tile_row0;  // [ntiles] first row (processing order)
  const int* __restrict__ tile_row1;  // [ntiles] one past the last row
  const int* __restrict__ tile_rec;   // [ntiles+1] record range of each tile
  const long long* __restrict__ rec_off;  // [nrec] byte offset in recbuf
  const int* __restrict__ rec_bytes;      // [nrec]
  const int* __restrict__ rec_flags;      // [nrec] kRecBarrier / kRecLong
  const unsigned char* __restrict__ recbuf;
  const int* __restrict__ long_col;
  const T* __restrict__ long_val;
  T* y;              // output, pre-filled with the sentinel
  unsigned* ticket;  // [0] next tile, [1] finished tiles, [2] exited blocks
  int* err;
  int tile_rows;
};

__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

// Counts a finished tile; true in the block that finished the last one.
// Thread 0 only, after the tile's partials are written.
__device__ __forceinline__ bool chunk_finished(unsigned* ticket, int nchunks) {
  __threadfence();
  return atomicAdd(&ticket[1], 1u) == (unsigned)nchunks - 1u;
}

// ------------------------------------------------------------ mbarrier / TMA
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait on an mbarrier phase; false on timeout / abort.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, int* err) {
  if (mbar_try_wait(b, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  const uint64_t budget = spin_budget(err);
  while (true) {
    if (mbar_try_wait(b, parity)) return true;
    if (ld_volatile(err) != 0 || globaltimer_ns() - t0 > budget) {
      atomicCAS(err, 0, (int)GB_TIMEOUT);
      return false;
    }
  }
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void named_barrier_consumers() {
  asm volatile("bar.sync 1, %0;" ::"n"(kTriConsumers * 32) : "memory");
}

template <typename T>
__device__ __forceinline__ T dep_value(const T* y, const T* sm, int c, int t0, int t1, int* err) {
  if (c >= t0 && c < t1) return sm[c - t0];
  return wait_value(y + c, err);
}

// Remote values of a thread's first row in the next record, read before the
// level barrier so that the dependency chain does not wait on L2.
constexpr int kTriPrefetchRemote = 2;
template <typename T>
struct RemotePrefetch {
  int col[kTriPrefetchRemote];
  T val[kTriPrefetchRemote];
};

template <typename T>
__device__ __forceinline__ void prefetch_remote(const TriArgs<T>& A, const unsigned char* rec, int t0,
                                                int t1, int ct, RemotePrefetch<T>& pf) {
#pragma unroll
  for (int q = 0; q < kTriPrefetchRemote; ++q) pf.col[q] = -1;
  const RecHdr h = *reinterpret_cast<const RecHdr*>(rec);
  if ((h.flags & kRecLong) || ct >= h.nrows) return;
  const int R4 = (h.nrows + 3) & ~3;
  const int* cols = reinterpret_cast<const int*>(rec + sizeof(RecHdr) + 4 * R4 + 2 * sizeof(T) * R4);
  int q = 0;
  for (int k = 0; k < h.len && q < kTriPrefetchRemote; ++k) {
    const int c = cols[k * R4 + ct];
    if (c < 0) break;
    if (c < t0 || c >= t1) {
      pf.col[q] = c;
      pf.val[q] = ld_relaxed(A.y + c);
      ++q;
    }
  }
}

// Solves the rows of one staged record (consumer threads ct = 0..127).
template <typename T, bool EXACT>
__device__ __forceinline__ void solve_record(const TriArgs<T>& A, T* sm, int t0, int t1,
                                             const unsigned char* rec, int ct,
                                             const RemotePrefetch<T>& pf) {
  const RecHdr h = *reinterpret_cast<const RecHdr*>(rec);
  const int R4 = (h.nrows + 3) & ~3;
  const int* rows = reinterpret_cast<const int*>(rec + sizeof(RecHdr));
  const T* diag = reinterpret_cast<const T*>(rows + R4);
  const T* dinv = diag + R4;
  if (h.flags & kRecLong) {
    // one row, the whole first consumer warp reduces it
    if (ct >= 32) return;
    const int row = rows[0];
    T acc = T(0);
    for (int k = ct; k < h.len; k += 32) {
      const int c = __ldg(A.long_col + h.off + k);
      acc = fma_rn(__ldg(A.long_val + h.off + k), dep_value(A.y, sm, c, t0, t1, A.err), acc);
    }
    acc = warp_sum(acc);
    if (ct == 0) {
      const T r = sub_rn(sm[row - t0], acc);
      const T yv = publishable(EXACT ? div_rn(r, diag[0]) : r * dinv[0]);
      sm[row - t0] = yv;
      st_relaxed(A.y + row, yv);
    }
    return;
  }
  const int* cols = reinterpret_cast<const int*>(dinv + R4);
  const T* vals = reinterpret_cast<const T*>(cols + (size_t)h.len * R4);
  for (int r = ct; r < h.nrows; r += kTriConsumers * 32) {
    const int row = rows[r];
    T acc = sm[row - t0];
    for (int k = 0; k < h.len; ++k) {
      const int c = cols[k * R4 + r];
      if (c < 0) break;
      const T l = vals[k * R4 + r];
      T v;
      if (c >= t0 && c < t1) {
        v = sm[c - t0];
      } else {
        v = sentinel<T>();
        if (r == ct) {
#pragma unroll
          for (int q = 0; q < kTriPrefetchRemote; ++q)
            if (pf.col[q] == c) v = pf.val[q];
        }
        if (is_sentinel(v)) v = wait_value(A.y + c, A.err);
      }
      acc = EXACT ? sub_rn(acc, mul_rn(l, v)) : fma_rn(-l, v, acc);
    }
    const T yv = publishable(EXACT ? div_rn(acc, diag[r]) : acc * dinv[r]);
    sm[row - t0] = yv;
    st_relaxed(A.y + row, yv);
  }
}

// Phase A / C loops: every thread first issues the loads of kTriUnroll rows
// (OP::pre / OP::dpre), then computes and stores them, so a tile's vector
// traffic streams instead of paying one DRAM round trip per row.
constexpr int kTriUnroll = 8;

template <typename T, typename OP>
__device__ __forceinline__ void phase_rhs(OP& op, T* sm, int t0, int t1) {
  for (int b = t0 + (int)threadIdx.x; b < t1; b += kTriUnroll * kTriThreads) {
    typename OP::Pre pr[kTriUnroll];
#pragma unroll
    for (int u = 0; u < kTriUnroll; ++u) {
      const int i = b + u * kTriThreads;
      if (i < t1) pr[u] = op.pre(i);
    }
#pragma unroll
    for (int u = 0; u < kTriUnroll; ++u) {
      const int i = b + u * kTriThreads;
      if (i < t1) sm[i - t0] = op.rhs(i, pr[u]);
    }
  }
}

template <typename T, typename OP>
__device__ __forceinline__ void phase_done(OP& op, const T* sm, int t0, int t1) {
  for (int b = t0 + (int)threadIdx.x; b < t1; b += kTriUnroll * kTriThreads) {
    typename OP::DPre pr[kTriUnroll];
#pragma unroll
    for (int u = 0; u < kTriUnroll; ++u) {
      const int i = b + u * kTriThreads;
      if (i < t1) pr[u] = op.dpre(i);
    }
#pragma unroll
    for (int u = 0; u < kTriUnroll; ++u) {
      const int i = b + u * kTriThreads;
      if (i < t1) op.done(i, sm[i - t0], pr[u]);
    }
  }
}

template <typename T, typename OP, bool EXACT>
__global__ void __launch_bounds__(kTriThreads) tri_tile_kernel(TriArgs<T> A, OP op) {
  extern __shared__ __align__(128) unsigned char tri_smem[];
  unsigned char* ring = tri_smem;                                   // kTriSlots x kTriSlotBytes
  T* sm = reinterpret_cast<T*>(tri_smem + kTriSlots * kTriSlotBytes);  // tile values
  __shared__ __align__(8) uint64_t full_bar[kTriSlots], empty_bar[kTriSlots];
  __shared__ long long s_roff[kTriRecTable];
  __shared__ int s_rbytes[kTriRecTable];
  __shared__ int s_rflags[kTriRecTable];
  __shared__ unsigned s_issued, s_consumed;
  __shared__ int s_tile;
  __shared__ double s_red[64];
  op.begin();
  if (!op.active()) {
    if (blockIdx.x == 0 && threadIdx.x == 0) op.inactive_end();
    return;  // no ticket touched
  }
  const int wid = threadIdx.x >> 5;
  const bool producer = wid == kTriConsumers;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kTriSlots; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], kTriConsumers);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  unsigned issued = 0;    // records issued by this CTA's producer (all tiles)
  unsigned consumed = 0;  // records consumed by this CTA's consumers
  bool failed = false;
  while (true) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(&A.ticket[0], 1u);
    __syncthreads();
    const int k = s_tile;
    __syncthreads();
    if (k >= A.ntiles) break;
    const int t0 = __ldg(A.tile_row0 + k), t1 = __ldg(A.tile_row1 + k);
    const int rec0 = __ldg(A.tile_rec + k), rec1 = __ldg(A.tile_rec + k + 1);
    // the tile's record table, so the producer issues copies back to back
    for (int q = threadIdx.x; q < rec1 - rec0 && q < kTriRecTable; q += kTriThreads) {
      s_roff[q] = __ldg(A.rec_off + rec0 + q);
      s_rbytes[q] = __ldg(A.rec_bytes + rec0 + q);
      s_rflags[q] = __ldg(A.rec_flags + rec0 + q);
    }
    // A) right-hand sides
    phase_rhs<T>(op, sm, t0, t1);
    __syncthreads();
    // B) records
    if (producer) {
      if ((threadIdx.x & 31) == 0) {
        for (int j = rec0; j < rec1 && !failed; ++j, ++issued) {
          const int slot = issued % kTriSlots;
          const unsigned use = issued / kTriSlots;
          if (!mbar_wait(&empty_bar[slot], (use & 1u) ^ 1u, A.err)) {
            failed = true;
            break;
          }
          const int q = j - rec0;
          const unsigned bytes = (unsigned)(q < kTriRecTable ? s_rbytes[q] : __ldg(A.rec_bytes + j));
          const long long off = q < kTriRecTable ? s_roff[q] : __ldg(A.rec_off + j);
          mbar_expect_tx(&full_bar[slot], bytes);
          tma_load_1d(ring + slot * kTriSlotBytes, A.recbuf + off, bytes, &full_bar[slot]);
        }
      }
      issued = __shfl_sync(0xffffffffu, issued, 0);
      failed = __shfl_sync(0xffffffffu, failed, 0);
    } else {
      const int ct = threadIdx.x;
      RemotePrefetch<T> pf;
#pragma unroll
      for (int q = 0; q < kTriPrefetchRemote; ++q) pf.col[q] = -1;
      for (int j = rec0; j < rec1; ++j, ++consumed) {
        const int slot = consumed % kTriSlots;
        const unsigned use = consumed / kTriSlots;
        if (!failed && !mbar_wait(&full_bar[slot], use & 1u, A.err)) failed = true;
        const unsigned char* rec = ring + slot * kTriSlotBytes;
        if (!failed) {
          solve_record<T, EXACT>(A, sm, t0, t1, rec, ct, pf);
        }
        __syncwarp();
        if ((ct & 31) == 0) mbar_arrive(&empty_bar[slot]);
        // if the next record is staged already, read its remote values now,
        // before the level barrier (never wait for it here)
#pragma unroll
        for (int q = 0; q < kTriPrefetchRemote; ++q) pf.col[q] = -1;
        if (!failed && j + 1 < rec1) {
          const unsigned nx = consumed + 1;
          if (mbar_try_wait(&full_bar[nx % kTriSlots], (nx / kTriSlots) & 1u))
            prefetch_remote(A, ring + (nx % kTriSlots) * kTriSlotBytes, t0, t1, ct, pf);
        }
        // level ends: every consumer warp reads the same table, so all take
        // the same barriers even if one of them gave up waiting for a record
        const int q = j - rec0;
        const int fl = q < kTriRecTable ? s_rflags[q] : __ldg(A.rec_flags + j);
        if (fl & kRecBarrier) named_barrier_consumers();
      }
    }
    __syncthreads();
    // C) epilogue
    phase_done<T>(op, sm, t0, t1);
    op.chunk_end(k, A.ntiles, A.ticket, s_red);
    __syncthreads();
  }
  // Drain: every issued copy has been consumed (consumers wait on each full
  // barrier, or fail only after the error word is set; in that case wait,
  // bounded, for the copies still in flight before the CTA's shared memory
  // goes away).
  if (threadIdx.x == 0) s_consumed = consumed;
  if (threadIdx.x == kTriConsumers * 32) s_issued = issued;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (unsigned u = s_consumed; u < s_issued; ++u) {
      const int slot = u % kTriSlots;
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&full_bar[slot], (u / kTriSlots) & 1u) &&
             globaltimer_ns() - t0 < kSpinBudgetNs) {
      }
    }
  }
  __syncthreads();
  // the last block to leave resets the counters for the next launch
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&A.ticket[2], 1u) == gridDim.x - 1u) {
      A.ticket[0] = 0u;
      A.ticket[1] = 0u;
      A.ticket[2] = 0u;
      __threadfence();
    }
  }
}

int tri_blocks_per_sm();

// Launches the tiled solve: dynamic shared memory = the record ring plus one
// tile of T values; a persistent grid of min(tiles, SMs x resident CTAs).
template <typename T, typename OP, bool EXACT>
int tri_launch(const TriPlan& p, const TriArgs<T>& A, OP op, cudaStream_t s) {
  if (p.ntiles <= 0) return GB_OK;
  const size_t smem = (size_t)kTriSlots * kTriSlotBytes + (size_t)p.tile_rows * sizeof(T);
  static bool attr_set = false;  // one per instantiation
  if (!attr_set) {
    GB_CUDA_TRY(cudaFuncSetAttribute(tri_tile_kernel<T, OP, EXACT>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tri_tile_kernel<T, OP, EXACT>,
                                                    kTriThreads, smem) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  per_sm = per_sm < tri_blocks_per_sm() ? per_sm : tri_blocks_per_sm();
  const long long cap = (long long)device_sm_count() * per_sm;
  const int grid = (int)(p.ntiles < cap ? p.ntiles : cap);
  tri_tile_kernel<T, OP, EXACT><<<grid, kTriThreads, smem, s>>>(A, op);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

template <typename T>
TriArgs<T> tri_args(const TriPlan& p, T* y, int* err);

// Plain solve: rhs from an input vector.
template <typename T>
struct OpPlain {
  const T* __restrict__ x;
  struct Pre {
    T x;
  };
  struct DPre {};
  __device__ __forceinline__ void begin() {}
  __device__ __forceinline__ bool active() const { return true; }
  __device__ __forceinline__ void inactive_end() {}
  __device__ __forceinline__ Pre pre(int r) const { return {x[r]}; }
  __device__ __forceinline__ T rhs(int, const Pre& p) const { return p.x; }
  __device__ __forceinline__ DPre dpre(int) const { return {}; }
  __device__ __forceinline__ void done(int, T, const DPre&) {}
  __device__ __forceinline__ void chunk_end(int, int nchunks, unsigned* ticket, double*) {
    if (threadIdx.x == 0) chunk_finished(ticket, nchunks);
  }
};

}  // namespace gb
