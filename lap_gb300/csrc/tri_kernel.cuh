// tri_kernel.cuh -- tiled sync-free sparse triangular solve, TMA-staged.
//
// Replaces cusparseDcsrsv2_solve (cuda_blas.cu:731-820, :500, :516).  Every
// row is solved as simple_lower/upper_triangular_solve (simple_blas.c:46-85)
// does: acc = rhs; acc -= l_ij * y_j in the row's column order; y_i = acc /
// d_i.  EXACT keeps that rounding (separate mul and sub, a true division);
// otherwise the row computes y_i = rhs/d_i - sum (l_ij/d_i) y_j with FMAs and
// the precomputed reciprocal of d_i, and does the scaling (and the terms
// whose y_j is already available) before it waits -- GB300 runs FP64 at 1/64
// of its FP32 rate, so every FP64 instruction on the dependency chain counts.
//
// Schedule (TriPlan, built on the host): rows are cut into contiguous tiles;
// inside a tile rows are ordered by their global level (dependency depth in
// the whole factor) and packed into RECORDS of at most 32 rows of one level (rows,
// diagonal, its reciprocal, dependency columns and values column-major;
// contiguous and 16-byte aligned).  The FP32 records of a plan whose rows all
// have at most kTriHeld dependencies use a fixed layout instead (one 48-byte
// block per row at a fixed offset), read by the short-record kernel only.
// One CTA solves one tile at a time:
//   * a producer warp streams the tile's records into a ring of shared-
//     memory slots with cp.async.bulk (TMA), one mbarrier per slot, several
//     lanes issuing copies in parallel;
//   * consumer warps take the records round-robin, one row per lane.  A
//     dependency inside the tile is read from the tile's solution array in
//     shared memory, spinning while it still holds the sentinel (or, in the
//     counter form, once the tile's earlier levels are counted complete);
//     one in an earlier tile is read from the inbox the previous tile's CTA
//     pushes into, from that CTA's array, or from global memory with
//     backoff, by the launch form.
//     There is no barrier between levels: a row waits exactly for its own
//     dependencies, so the wavefront advances at shared-memory latency.
//     A row's right-hand side is loaded before its dependencies are awaited.
// Progress: a record only depends on earlier records, the earliest
// unfinished record always has its inputs, and the ring always holds it; a
// tile only depends on earlier tiles, taken by ticket by running CTAs.
// Every wait is bounded in wall-clock time; on expiry the error word is set,
// waiters release their dependents with a NaN and the CTA drains its own
// copies before leaving.
//
// OP contract (right-hand side and epilogue of each solved row):
//   void begin();  bool active();  void inactive_end()   (block 0, !active)
//   Pre pre(int row)                loads of the rhs (issued early, up to one
//                                   record ahead: they may read only data
//                                   written before the launch)
//   T rhs(int row, const Pre&)      rhs value (may store updated vectors)
//   DPre dpre(int row)              loads for the epilogue (same rule)
//   void done(int row, T y, const DPre&)
//   void prefetch(int r0, int r1, int part)   producer lane `part` (of
//        kTriProdLanes), once per tile: L2 prefetch of its share of the
//        vectors pre()/dpre() read over the tile's rows [r0, r1)
//   void chunk_end(tile_ix, ntiles, ticket, sm)   whole block, after the
//        tile; ticket[1] counts finished tiles (chunk_finished()).
#pragma once

#include <type_traits>

#include "gb_common.cuh"
#include "kernels.h"
#include "spmv_bundle.cuh"

namespace gb {

// Consumer warps per CTA.  FP64 solves use 8: GB300 issues one FP64 lane op
// per two cycles per SM sub-partition, so more warps only queue their FP64
// work in front of the dependency chain.  FP32 solves have no such limit and
// use 15: with the producer that is 16 warps, 4 per SM sub-partition, which
// leaves 128 registers a thread (a 17-warp block is capped at 96, and the
// record code then spills around its waits).
#ifndef GB_TRI_CONSUMERS32
#define GB_TRI_CONSUMERS32 15
#endif
// 1: a consumer warp issues the right-hand-side loads of its next record
// (pre / dpre) as soon as that record has landed in the ring, while it
// solves the current one, so a record's L2 round trip for its rhs is off
// the warp's serial path.
#ifndef GB_TRI_RHS_AHEAD
#define GB_TRI_RHS_AHEAD 1
#endif
// The short-record kernel (SHORT below) has its own counts.  FP32: 13 (128^3
// split PCG with the fixed-layout records and polling solves: 119.8 ms
// against 121.0 with 15 and 123.0 with 17; 11, 19, 23 and 31 measured slower
// earlier).
// FP64: 12 (128^3 FP64 lower / upper 298 / 339 us; 8 warps 321 / 364, 15
// warps 308 / 340): its records are short enough that more warps in flight
// outweigh the queueing on the FP64 pipe.
#ifndef GB_TRI_CONSUMERS32S
#define GB_TRI_CONSUMERS32S 13
#endif
#ifndef GB_TRI_CONSUMERS64S
#define GB_TRI_CONSUMERS64S 12
#endif
template <typename T, bool SHORT = false>
struct TriCons {
  static constexpr int n = sizeof(T) == 8 ? (SHORT ? GB_TRI_CONSUMERS64S : 8)
                                          : (SHORT ? GB_TRI_CONSUMERS32S : GB_TRI_CONSUMERS32);
  static constexpr int threads = (n + 1) * 32;  // + one producer warp
};
constexpr int kTriSlots = 40;                          // ring depth (records in flight)
constexpr int kTriSlotBytes = 2048;                    // max record size
constexpr int kTriL2Ahead = 32;                        // records prefetched into L2 ahead of the ring
constexpr int kTriProdLanes = 8;                       // producer lanes issuing copies in parallel
static_assert(kTriSlots % kTriProdLanes == 0, "a slot is always refilled by the same producer lane");
constexpr int kTriRecTable = 1024;                     // records of a tile cached in smem
constexpr int kTriMaxDynSmem = 212 * 1024;             // ring + the largest tile (FP32 x 32768 rows)
constexpr int kTriRecRows = 32;                        // rows per record (one per lane)
constexpr int kRecLong = 2;                            // record flag: one row, warp-reduced
// A row of more than two parts' dependencies (a power-law hub; a part is
// kTriPartDeps entries unless the plan is told otherwise) is split: PART
// records reduce a part of its entries each (any warp) into a slot, and a
// COMBINE record after them adds the slots in a fixed order and solves the
// row.  Header: off = the part's first long entry, pad1 = its slot (the
// combine's first slot), len = the part's entries (the combine's parts).
constexpr int kRecPart = 4;
constexpr int kRecCombine = 8;
constexpr int kTriPartDeps = 1024;

// Record header (32 bytes).  Layout after it, R4 = nrows rounded up to 4:
//   int rows[R4]; T diag[R4]; T dinv[R4]; int cols[len*R4]; T vals[len*R4]
// (LONG records: no cols/vals; they live at long_col/long_val[off ...]).
// wait_for = number of the tile's records in earlier tile-levels: the record
// may start once that many records of the tile are complete.  pad0 = the
// record's index in the plan, which a consumer checks in the staged copy.
struct RecHdr {
  int nrows, len, flags, off, wait_for, pad0, pad1, pad2;
};
constexpr int kRecHdrBytes = (int)sizeof(RecHdr);
static_assert(kRecHdrBytes == 32, "record header layout");

// Fixed layout of the FP32 records of a short-only plan (TriPlan::fixed32):
// a 16-byte header {nrows, wait_for, record index, kFixTag} and one 48-byte block
// per row (lane), three 16-byte words
//   {row, c0, c1, c2} {c3, 1/d, l0/d, l1/d} {l2/d, l3/d, 0, 0}
// (c_k = -1 past the row's dependencies).  Every offset is fixed, so a lane
// issues all of its record's loads at once, with the header's beside them.
constexpr int kFixHdrBytes = 16;
constexpr int kFixLaneBytes = 48;
// layout tag in the header, checked with the record index once a record is
// solved (the general layout has a short record's entry offset, 0, there);
// the launcher runs the fixed-layout kernel only on plans in that layout
constexpr int kFixTag = 0x31584946;
static_assert(kFixHdrBytes + 32 * kFixLaneBytes <= 2048, "a fixed record fits a ring slot");

template <typename T>
struct TriArgs {
  int ntiles;
  const int* __restrict__ tile_row0;  // [ntiles] first row (processing order)
  const int* __restrict__ tile_row1;  // [ntiles] one past the last row
  const int* __restrict__ tile_rec;   // [ntiles+1] record range of each tile
  const long long* __restrict__ rec_off;  // [nrec] byte offset in recbuf
  const int* __restrict__ rec_bytes;      // [nrec]
  const unsigned char* __restrict__ recbuf;
  const int* __restrict__ long_col;
  const T* __restrict__ long_val;
  T* y;              // output, pre-filled with the sentinel
  unsigned* ticket;  // [0] next tile, [1] finished tiles, [2] exited blocks
  int* err;
  int tile_rows;
  T* part;   // [plan nslots] partial sums of split rows (sentinel between uses)
  int poll;  // the plan's levels hold several records: lower solves poll values (see op_polls_values)
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
// Bounded wait until the producer has issued stream record u into its slot
// (s_last_u[slot] == u); false on timeout / abort.  A consumer waits for this
// before the slot's full barrier: the barrier's parity names a phase only
// within one lap of the ring, and a consumer can reach record u while the
// slot still holds record u - 2 * kTriSlots (its owner lags), whose phase has
// the same parity.
__device__ __forceinline__ bool wait_issued(const unsigned* last_u, unsigned u, int* err) {
  if (*(const volatile unsigned*)last_u == u) return true;
  SpinClock clk;
  for (unsigned polls = 1;; ++polls) {
    if (*(const volatile unsigned*)last_u == u) return true;
    if ((polls & 63u) == 0u && clk.expired(err)) return false;
  }
}
// Bounded wait on an mbarrier phase; false on timeout / abort.  The clock
// and the (global) error word are checked only every 64 polls so that a
// satisfied barrier is noticed at shared-memory speed.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, int* err) {
  if (mbar_try_wait(b, parity)) return true;
  SpinClock clk;
  for (unsigned polls = 1;; ++polls) {
    if (mbar_try_wait(b, parity)) return true;
    if ((polls & 63u) == 0u && clk.expired(err)) return false;
  }
}
__device__ __forceinline__ void tma_prefetch_l2(const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// L2 prefetch of piece `part` of `nparts` of v[r0 .. r1): a hint, so the
// range is shrunk to whole 16-byte units inside it (the bulk prefetch's
// alignment rule) and never reaches outside the rows asked for.
template <typename T>
__device__ __forceinline__ void prefetch_rows_l2(const T* v, int r0, int r1, int part, int nparts) {
  if (v == nullptr || r1 <= r0) return;
  const uintptr_t a = ((uintptr_t)(v + r0) + 15u) & ~(uintptr_t)15u;
  const uintptr_t b = (uintptr_t)(v + r1) & ~(uintptr_t)15u;
  if (b <= a) return;
  const uintptr_t piece = (((b - a) + nparts - 1) / nparts + 15u) & ~(uintptr_t)15u;
  const uintptr_t s0 = a + (uintptr_t)part * piece;
  if (s0 >= b) return;
  const uintptr_t n = (b - s0) < piece ? (b - s0) : piece;
  tma_prefetch_l2(reinterpret_cast<const void*>(s0), (unsigned)n);
}

// Spin on a tile-local value in shared memory (written by another warp of
// this CTA).  Bounded like the global waits.  The spin loops are kept out of
// line so that the unrolled row code stays small; only the first read is
// inlined.
template <typename T>
__device__ __noinline__ T wait_local_slow(const T* p, int* err) {
  const volatile T* vp = p;
  SpinClock clk;
  for (unsigned polls = 1;; ++polls) {
    const T v = *vp;
    if (!is_sentinel(v)) return v;
    if ((polls & 255u) == 0u && clk.expired(err)) return (T)__int_as_float(0x7FC00000);
  }
}
template <typename T>
__device__ __forceinline__ T wait_local(const T* p, int* err) {
  const T v = *(const volatile T*)p;
  return is_sentinel(v) ? wait_local_slow(p, err) : v;
}
template <typename T>
__device__ __noinline__ T wait_value_slow(const T* p, int* err) {
  return wait_value(p, err);
}

template <typename T>
__device__ __forceinline__ T dep_value(const TriArgs<T>& A, const T* sy, int c, int t0, int t1) {
  if (c >= t0 && c < t1) return wait_local(sy + (c - t0), A.err);
  const T v = ld_relaxed(A.y + c);
  return is_sentinel(v) ? wait_value_slow(A.y + c, A.err) : v;
}

__device__ __forceinline__ void st_shared_volatile(double* p, double v) { *(volatile double*)p = v; }
__device__ __forceinline__ void st_shared_volatile(float* p, float v) { *(volatile float*)p = v; }

// Tile-local completion counter: release by the finishing warp, acquire by
// the waiting one (shared memory, CTA scope -- no full fence needed).
__device__ __forceinline__ int ld_acquire_cta(const int* p) {
  int v;
  asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_cta_add(int* p, int v) {
  asm volatile("red.release.cta.shared::cta.add.s32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}

// Waits (warp-uniform) until `need` records of the current tile are
// complete, i.e. every earlier tile-level of this record is done.
static __device__ __noinline__ void wait_level_slow(const int* s_done, int need, int* err) {
  SpinClock clk;
  for (unsigned polls = 1;; ++polls) {
    if (ld_acquire_cta(s_done) >= need) return;
    if ((polls & 255u) == 0u && clk.expired(err)) return;
  }
}
__device__ __forceinline__ void wait_level(const int* s_done, int need, int* err) {
  if (need <= 0) return;
  // every lane polls the same word (a broadcast read): no warp sync needed
  if (ld_acquire_cta(s_done) < need) wait_level_slow(s_done, need, err);
}

// Solves one staged record with one warp (lane = row of the record; a LONG
// record's single row is split across the warp).  Everything that does not
// depend on the record's inputs is done before the wait: the rhs (its loads
// and FP64 vector updates), the record's indices and values, the early reads
// of other tiles' values.  After the wait only the tile-local values are
// read (one round of shared-memory loads) and the FMA chain runs; the
// completion is published before the global stores.
constexpr int kTriHeld = 4;       // dependencies held in registers per row
constexpr int kTriTailBatch = 8;  // loads in flight per row beyond the held ones
constexpr int kTriLongBatch = 8;  // loads in flight per lane in a LONG record

// Link of a tile to its neighbours inside a thread-block cluster: `in` is
// this CTA's inbox (shared memory) holding the previous tile's rows
// [in0, in1), pushed there by the CTA that solves them; `out` is the
// shared::cluster address of the next CTA's inbox (0: none).  Without a
// cluster both are empty and every other-tile value comes through L2.
//
// FP64 tiles leave no room for an inbox; their clusters PULL instead:
// `in_remote` is the shared::cluster address of the previous tile's own
// solution array in its CTA, polled there (sentinel as flag).
template <typename T>
struct TriLink {
  const T* in = nullptr;
  int in0 = 0, in1 = 0;
  uint32_t out = 0;
  uint32_t in_remote = 0;
};

__device__ __forceinline__ float ld_cluster_relaxed(uint32_t addr, float*) {
  float v;
  asm volatile("ld.relaxed.cluster.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ double ld_cluster_relaxed(uint32_t addr, double*) {
  double v;
  asm volatile("ld.relaxed.cluster.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}
// Polls a value in another CTA of the cluster; bounded like every wait.
template <typename T>
__device__ __noinline__ T wait_remote_slow(uint32_t addr, int* err) {
  SpinClock clk;
  for (unsigned polls = 1;; ++polls) {
    const T v = ld_cluster_relaxed(addr, (T*)nullptr);
    if (!is_sentinel(v)) return v;
    if ((polls & 255u) == 0u && clk.expired(err)) return (T)__int_as_float(0x7FC00000);
  }
}

__device__ __forceinline__ void st_cluster(uint32_t addr, float v) {
  asm volatile("st.relaxed.cluster.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(uint32_t addr, double v) {
  asm volatile("st.relaxed.cluster.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}

// A value of another tile: from the inbox when the previous tile pushes it
// there, else from global memory (sentinel while not yet solved).
template <typename T>
__device__ __forceinline__ T other_tile_read(const TriArgs<T>& A, const TriLink<T>& L, int c) {
  if (L.in && c >= L.in0 && c < L.in1) return *(const volatile T*)(L.in + (c - L.in0));
  if (L.in_remote && c >= L.in0 && c < L.in1)
    return ld_cluster_relaxed(L.in_remote + (uint32_t)(c - L.in0) * (uint32_t)sizeof(T), (T*)nullptr);
  return ld_relaxed(A.y + c);
}
template <typename T>
__device__ __forceinline__ T other_tile_wait(const TriArgs<T>& A, const TriLink<T>& L, int c) {
  if (L.in && c >= L.in0 && c < L.in1) return wait_local_slow(L.in + (c - L.in0), A.err);
  if (L.in_remote && c >= L.in0 && c < L.in1)
    return wait_remote_slow<T>(L.in_remote + (uint32_t)(c - L.in0) * (uint32_t)sizeof(T), A.err);
  return wait_value_slow(A.y + c, A.err);
}

// An OP with `static constexpr bool kPollValues = true` has its rows read
// their tile-local dependencies by polling the values (sentinel as flag)
// instead of first waiting for every earlier tile-level to be counted
// complete -- when the plan's levels hold several records each (A.poll):
// no release/acquire pair on the chain, but every lane polls its own
// addresses.  Measured: the 128^3 lower solve 284 vs 308 us; where a level
// is one record (8-row tiles of a 1024^2 grid) 1522 vs 1052 us, so such
// plans keep the counter; upper solves keep it everywhere (128^3: 480 vs
// 373 us).
template <typename OP, typename = void>
struct op_polls_values : std::false_type {};
template <typename OP>
struct op_polls_values<OP, std::void_t<decltype(OP::kPollValues)>> : std::bool_constant<OP::kPollValues> {};

// The row a lane solves in a staged record (-1: idle lane).
__device__ __forceinline__ int record_row(const unsigned char* rec, int lane) {
  const RecHdr* h = reinterpret_cast<const RecHdr*>(rec);
  const bool lng = (h->flags & kRecLong) != 0;
  const int* rows = reinterpret_cast<const int*>(rec + sizeof(RecHdr));
  return (lng || lane < h->nrows) ? rows[lng ? 0 : lane] : -1;
}

// Right-hand-side loads of a record issued ahead of it (have: they were).
template <typename OP>
struct RhsAhead {
  typename OP::Pre pr;
  typename OP::DPre dp;
  bool have = false;
};

// The row a lane solves in a staged fixed-layout record (-1: idle lane).
__device__ __forceinline__ int record_row_fixed(const unsigned char* rec, int lane) {
  const int nrows = *reinterpret_cast<const int*>(rec);
  const int row = *reinterpret_cast<const int*>(rec + kFixHdrBytes + lane * kFixLaneBytes);
  return lane < nrows ? row : -1;
}
// The index a staged record carries, or -1 for a fixed-layout kernel handed
// a record without the layout's tag.
__device__ __forceinline__ int record_index(const unsigned char* rec, bool fixed) {
  const int* h = reinterpret_cast<const int*>(rec);
  return fixed ? (h[3] == kFixTag ? h[2] : -1) : reinterpret_cast<const RecHdr*>(rec)->pad0;
}

// SHORT: the plan has only short records of at most kTriHeld dependencies
// (grids, kNN graphs): the long-row, hub-part, combine and tail paths are
// compiled out, which halves the kernel's code.
template <typename T, bool EXACT, bool POLL, typename OP, bool SHORT = false>
__device__ __forceinline__ void solve_record(const TriArgs<T>& A, OP& op, T* sy, int t0, int t1,
                                             const unsigned char* rec, int lane, int* s_done,
                                             const TriLink<T>& L, const RhsAhead<OP>& ahead) {
  const RecHdr h = *reinterpret_cast<const RecHdr*>(rec);
  const int R4 = (h.nrows + 3) & ~3;
  const int* rows = reinterpret_cast<const int*>(rec + sizeof(RecHdr));
  const T* diag = reinterpret_cast<const T*>(rows + R4);
  const T* dinv = diag + R4;
  const bool lng = !SHORT && (h.flags & kRecLong) != 0;
  const bool act = lng ? true : lane < h.nrows;
  const int row = act ? rows[lng ? 0 : lane] : -1;
  typename OP::Pre pr;
  typename OP::DPre dp;
  if (act) {
    if (ahead.have) {
      pr = ahead.pr;
      dp = ahead.dp;
    } else {
      pr = op.pre(row);
      dp = op.dpre(row);
    }
  }
  const int* cols = reinterpret_cast<const int*>(dinv + R4);
  const T* vals = reinterpret_cast<const T*>(cols + (size_t)h.len * R4);
  int hc[kTriHeld];
  T hl[kTriHeld], hv[kTriHeld];
  const bool short_act = !lng && act;
#pragma unroll
  for (int k = 0; k < kTriHeld; ++k) {
    hc[k] = -1;
    hv[k] = sentinel<T>();
    hl[k] = T(0);
    if (short_act && k < h.len) {
      const int c = cols[k * R4 + lane];
      hc[k] = c;
      if (c >= 0) {
        hl[k] = vals[k * R4 + lane];
        if (c < t0 || c >= t1) hv[k] = other_tile_read(A, L, c);  // other tile: read early
      }
    }
  }
  const T dg = short_act ? (EXACT ? diag[lane] : dinv[lane]) : T(0);
  T acc = T(0);
  if (act && (!lng || lane == 0)) acc = op.rhs(row, pr);
  bool pend[kTriHeld];
#pragma unroll
  for (int k = 0; k < kTriHeld; ++k) pend[k] = hc[k] >= 0;
  if (!EXACT && short_act) {
    // FMA-form records hold l/d: y = rhs/d - sum (l/d) y_dep.  The scaling
    // and the held dependencies in earlier tiles (read early; complete or
    // awaited here, independent of this tile's progress) leave the chain that
    // runs after the wait.  The order -- other tiles' terms first, then this
    // tile's, each in column order -- does not depend on timing, so results
    // are reproducible.
    acc = acc * dg;
#pragma unroll
    for (int k = 0; k < kTriHeld; ++k) {
      if (pend[k] && (hc[k] < t0 || hc[k] >= t1)) {
        const T v = is_sentinel(hv[k]) ? other_tile_wait(A, L, hc[k]) : hv[k];
        acc = fma_rn(-hl[k], v, acc);
        pend[k] = false;
      }
    }
  }
  // a tile-local value: complete once its level is counted, or polled
  auto local = [&](int c) -> T {
    if constexpr (POLL) return wait_local(sy + (c - t0), A.err);
    else return sy[c - t0];
  };
  if constexpr (!POLL) wait_level(s_done, h.wait_for, A.err);
  T yv = T(0);
  if (lng) {
    // lane-strided over the row; each lane issues kTriLongBatch loads before
    // it consumes them (same per-lane order as one at a time), and the next
    // batch's indices and values are in flight while this batch's values
    // are awaited: a power-law hub row has tens of thousands of entries
    T s = T(0);
    const bool part = (h.flags & kRecPart) != 0, comb = (h.flags & kRecCombine) != 0;
    if (comb) {
      // a split row: its parts' sums (written by other warps), lane-strided
      // and then the warp's fixed shuffle order, so the sum does not depend
      // on which part finished first; all of a lane's loads are in flight
      // before it waits on one
      T pv[kTriLongBatch];
#pragma unroll
      for (int u = 0; u < kTriLongBatch; ++u) {
        const int k = lane + 32 * u;
        pv[u] = k < h.len ? ld_relaxed(A.part + h.pad1 + k) : T(0);
      }
#pragma unroll
      for (int u = 0; u < kTriLongBatch; ++u) {
        const int k = lane + 32 * u;
        if (k < h.len) {
          T v = pv[u];
          if (is_sentinel(v)) v = wait_value_slow(A.part + h.pad1 + k, A.err);
          s = add_rn(s, v);
        }
      }
      for (int k = lane + 32 * kTriLongBatch; k < h.len; k += 32) {
        T v = ld_relaxed(A.part + h.pad1 + k);
        if (is_sentinel(v)) v = wait_value_slow(A.part + h.pad1 + k, A.err);
        s = add_rn(s, v);
      }
      s = warp_sum(s);
    } else {
    int cn[kTriLongBatch];
    T ln[kTriLongBatch];
#pragma unroll
    for (int u = 0; u < kTriLongBatch; ++u) {
      const int k = lane + 32 * u;
      cn[u] = k < h.len ? __ldg(A.long_col + h.off + k) : -1;
      ln[u] = cn[u] >= 0 ? __ldg(A.long_val + h.off + k) : T(0);
    }
    for (int k0 = lane; k0 < h.len; k0 += 32 * kTriLongBatch) {
      int cb[kTriLongBatch];
      T lb[kTriLongBatch], vb[kTriLongBatch];
#pragma unroll
      for (int u = 0; u < kTriLongBatch; ++u) {
        cb[u] = cn[u];
        lb[u] = ln[u];
        vb[u] = cb[u] < 0 ? T(0) : (cb[u] >= t0 && cb[u] < t1) ? local(cb[u]) : other_tile_read(A, L, cb[u]);
      }
#pragma unroll
      for (int u = 0; u < kTriLongBatch; ++u) {  // the next batch's indices, in flight meanwhile
        const int k = k0 + 32 * kTriLongBatch + 32 * u;
        cn[u] = k < h.len ? __ldg(A.long_col + h.off + k) : -1;
        ln[u] = cn[u] >= 0 ? __ldg(A.long_val + h.off + k) : T(0);
      }
#pragma unroll
      for (int u = 0; u < kTriLongBatch; ++u) {
        if (cb[u] < 0) continue;
        T v = vb[u];
        if ((cb[u] < t0 || cb[u] >= t1) && is_sentinel(v)) v = other_tile_wait(A, L, cb[u]);
        s = fma_rn(lb[u], v, s);
      }
    }
    s = warp_sum(s);
    }
    if (lane == 0 && part) {
      st_relaxed(A.part + h.pad1, publishable(s));  // this part's sum, for the combine record
    } else if (lane == 0) {
      const T r = sub_rn(acc, s);
      yv = publishable(EXACT ? div_rn(r, diag[0]) : r * dinv[0]);
      if (row >= t0 && row < t1) st_shared_volatile(sy + (row - t0), yv);  // the levels form has no tile rows
    }
  } else if (act) {
    // tile-local values: complete (earlier tile-levels) or polled; all loads at once
#pragma unroll
    for (int k = 0; k < kTriHeld; ++k)
      if (pend[k] && hc[k] >= t0 && hc[k] < t1) hv[k] = local(hc[k]);
    // the reference's order: acc = rhs; acc -= l_k * y_k for k ascending
#pragma unroll
    for (int k = 0; k < kTriHeld; ++k) {
      if (pend[k]) {
        T v = hv[k];
        if (is_sentinel(v)) v = other_tile_wait(A, L, hc[k]);  // other tile, not yet written
        acc = EXACT ? sub_rn(acc, mul_rn(hl[k], v)) : fma_rn(-hl[k], v, acc);
      }
    }
    // the rest of the row, kTriTailBatch dependencies at a time: all their
    // loads are issued before the first is consumed (a power-law row has
    // dozens, each an L2 round trip), then the terms are added in column
    // order; padding columns (-1) end the row
    for (int k0 = kTriHeld; !SHORT && k0 < h.len; k0 += kTriTailBatch) {
      int cb[kTriTailBatch];
      T lb[kTriTailBatch], vb[kTriTailBatch];
#pragma unroll
      for (int u = 0; u < kTriTailBatch; ++u) {
        const int k = k0 + u;
        cb[u] = k < h.len ? cols[k * R4 + lane] : -1;
        lb[u] = cb[u] >= 0 ? vals[k * R4 + lane] : T(0);
        vb[u] = cb[u] < 0 ? T(0) : (cb[u] >= t0 && cb[u] < t1) ? local(cb[u]) : other_tile_read(A, L, cb[u]);
      }
#pragma unroll
      for (int u = 0; u < kTriTailBatch; ++u) {
        if (cb[u] < 0) continue;
        T v = vb[u];
        if ((cb[u] < t0 || cb[u] >= t1) && is_sentinel(v)) v = other_tile_wait(A, L, cb[u]);
        acc = EXACT ? sub_rn(acc, mul_rn(lb[u], v)) : fma_rn(-lb[u], v, acc);
      }
    }
    yv = publishable(EXACT ? div_rn(acc, dg) : acc);
    if (row >= t0 && row < t1) st_shared_volatile(sy + (row - t0), yv);  // the levels form has no tile rows
  }
  __syncwarp();
  // the tile-level counter is read only where rows wait on whole levels
  if constexpr (!POLL)
    if (lane == 0) red_release_cta_add(s_done, 1);
  if (act && (!lng || lane == 0) && !(h.flags & kRecPart)) {
    if (L.out) st_cluster(L.out + (uint32_t)(row - t0) * (uint32_t)sizeof(T), yv);  // next tile's inbox
    st_relaxed(A.y + row, yv);
    op.done(row, yv, dp);
  }
}

// A fixed-layout FP32 record (FMA form, at most kTriHeld dependencies per
// row): the same arithmetic, in the same order, as solve_record's short
// path -- y = rhs/d, minus the other tiles' terms, then the tile's, each in
// column order -- with the header, row, columns, 1/d and values in four
// independent shared-memory loads.
// other_tile_wait with its spin inline (the value was read once already).
// The counter-waiting (upper) solves use these inline waits: 128^3 upper
// 273 -> 267 us; the polling (lower) solves keep the out-of-line ones (205
// against 208 us inline).
__device__ __forceinline__ float other_tile_wait_inline(const TriArgs<float>& A, const TriLink<float>& L, int c) {
  const bool inbox = L.in && c >= L.in0 && c < L.in1;
  const bool remote = !inbox && L.in_remote && c >= L.in0 && c < L.in1;
  if (!inbox && !remote) return wait_value_slow(A.y + c, A.err);  // global memory keeps its backoff
  SpinClock clk;
  for (unsigned polls = 1;; ++polls) {
    const float v = inbox ? *(const volatile float*)(L.in + (c - L.in0))
                          : ld_cluster_relaxed(L.in_remote + (uint32_t)(c - L.in0) * 4u, (float*)nullptr);
    if (!is_sentinel(v)) return v;
    if ((polls & 255u) == 0u && clk.expired(A.err)) return __int_as_float(0x7FC00000);
  }
}
__device__ __forceinline__ void wait_level_inline(const int* s_done, int need, int* err) {
  if (need <= 0 || ld_acquire_cta(s_done) >= need) return;
  SpinClock clk;
  for (unsigned polls = 1;; ++polls) {
    if (ld_acquire_cta(s_done) >= need) return;
    if ((polls & 255u) == 0u && clk.expired(err)) return;
  }
}

template <bool POLL, typename OP>
__device__ __forceinline__ void solve_record_fixed(const TriArgs<float>& A, OP& op, float* sy, int t0, int t1,
                                                   const unsigned char* rec, int lane, int* s_done,
                                                   const TriLink<float>& L, const RhsAhead<OP>& ahead) {
  const int4 hd = *reinterpret_cast<const int4*>(rec);
  const int4* lb = reinterpret_cast<const int4*>(rec + kFixHdrBytes + lane * kFixLaneBytes);
  const int4 b0 = lb[0], b1 = lb[1], b2 = lb[2];
  const bool act = lane < hd.x;
  const int row = b0.x;
  typename OP::Pre pr;
  typename OP::DPre dp;
  if (act) {
    if (ahead.have) {
      pr = ahead.pr;
      dp = ahead.dp;
    } else {
      pr = op.pre(row);
      dp = op.dpre(row);
    }
  }
  const int hc[kTriHeld] = {b0.y, b0.z, b0.w, b1.x};
  const float hl[kTriHeld] = {__int_as_float(b1.z), __int_as_float(b1.w), __int_as_float(b2.x),
                              __int_as_float(b2.y)};
  float hv[kTriHeld];
  bool pend[kTriHeld];
#pragma unroll
  for (int k = 0; k < kTriHeld; ++k) {
    pend[k] = act && hc[k] >= 0;
    hv[k] = sentinel<float>();
    if (pend[k] && (hc[k] < t0 || hc[k] >= t1)) hv[k] = other_tile_read(A, L, hc[k]);  // other tile: read early
  }
  float acc = 0.0f;
  if (act) acc = op.rhs(row, pr) * __int_as_float(b1.y);
#pragma unroll
  for (int k = 0; k < kTriHeld; ++k) {
    if (pend[k] && (hc[k] < t0 || hc[k] >= t1)) {
      const float v = !is_sentinel(hv[k]) ? hv[k]
                      : POLL      ? other_tile_wait(A, L, hc[k])
                                  : other_tile_wait_inline(A, L, hc[k]);
      acc = fma_rn(-hl[k], v, acc);
      pend[k] = false;
    }
  }
  if constexpr (POLL) {
    // The tile's values still pending, polled together in one inline loop
    // (bounded like every wait): waiting on them one after another through
    // an out-of-line spin took the 128^3 lower solve 218 us against 201-205.
    // Polling the inbox's values in the same loop measured 285 us.
#pragma unroll
    for (int k = 0; k < kTriHeld; ++k)
      if (pend[k]) hv[k] = *(const volatile float*)(sy + (hc[k] - t0));
    bool miss = false;
#pragma unroll
    for (int k = 0; k < kTriHeld; ++k) miss |= pend[k] && is_sentinel(hv[k]);
    if (miss) {
      SpinClock clk;
      for (unsigned polls = 1; miss; ++polls) {
        miss = false;
#pragma unroll
        for (int k = 0; k < kTriHeld; ++k)
          if (pend[k] && is_sentinel(hv[k])) {
            hv[k] = *(const volatile float*)(sy + (hc[k] - t0));
            miss |= is_sentinel(hv[k]);
          }
        if (miss && (polls & 255u) == 0u && clk.expired(A.err)) {  // gave up: NaN, as the other waits
#pragma unroll
          for (int k = 0; k < kTriHeld; ++k)
            if (pend[k] && is_sentinel(hv[k])) hv[k] = __int_as_float(0x7FC00000);
          miss = false;
        }
      }
    }
  } else {
    wait_level_inline(s_done, hd.y, A.err);  // every earlier tile-level complete
#pragma unroll
    for (int k = 0; k < kTriHeld; ++k)
      if (pend[k]) hv[k] = sy[hc[k] - t0];  // the tile's only: the other tiles' are folded
  }
#pragma unroll
  for (int k = 0; k < kTriHeld; ++k)
    if (pend[k]) acc = fma_rn(-hl[k], hv[k], acc);
  const float yv = publishable(acc);
  if (act && row >= t0 && row < t1) st_shared_volatile(sy + (row - t0), yv);  // the levels form has no tile rows
  __syncwarp();
  if constexpr (!POLL)
    if (lane == 0) red_release_cta_add(s_done, 1);
  if (act) {
    if (L.out) st_cluster(L.out + (uint32_t)(row - t0) * (uint32_t)sizeof(float), yv);  // next tile's inbox
    st_relaxed(A.y + row, yv);
    op.done(row, yv, dp);
  }
}

// ------------------------------------------------------------ clusters
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Every thread of every CTA of the cluster: release before, acquire after.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
// shared::cluster address of `p` (a shared-memory object of this CTA) in the
// CTA of the given rank
__device__ __forceinline__ uint32_t cluster_map(const void* p, unsigned rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ int ld_cluster_s32(uint32_t addr) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}

// CL = 1: one CTA per tile, tiles by ticket, every other-tile value through
// L2.  CL > 1 (FP32): a thread-block cluster of CL CTAs takes CL consecutive
// tiles (one group) per ticket, CTA rank r solving tile CL*g + r; each CTA
// keeps an inbox of the previous tile's values in its shared memory, which
// that tile's CTA fills with distributed-shared-memory stores as it solves
// rows, so the dependency that crosses a tile boundary inside the group
// costs a shared-memory poll instead of an L2 round trip.  Cluster barriers
// per group: after the group is known, after every inbox holds the
// sentinel (before any push), and at the end (no CTA refills or frees its
// inbox while its predecessor may still push into it).
template <typename T, typename OP, bool EXACT, int CL = 1, bool PULL = false, bool POLL = false,
          bool SHORT = false>
__global__ void __launch_bounds__((TriCons<T, SHORT>::threads), 1) tri_tile_kernel(TriArgs<T> A, OP op) {
  constexpr int kTriConsumers = TriCons<T, SHORT>::n;
  constexpr int kTriThreads = TriCons<T, SHORT>::threads;
  // short FP32 plans keep their FP32 records in the fixed layout (FMA form)
  constexpr bool kFixed = SHORT && sizeof(T) == 4;
  static_assert(!kFixed || !EXACT, "fixed-layout FP32 records hold the FMA form");
  extern __shared__ __align__(128) unsigned char tri_smem[];
  unsigned char* ring = tri_smem;                                     // kTriSlots x kTriSlotBytes
  T* sy = reinterpret_cast<T*>(tri_smem + kTriSlots * kTriSlotBytes);  // tile solution
  T* inbox = sy + A.tile_rows;  // CL > 1: the previous tile's values
  __shared__ __align__(8) uint64_t full_bar[kTriSlots], empty_bar[kTriSlots];
  __shared__ long long s_roff[kTriRecTable];
  __shared__ int s_rbytes[kTriRecTable];
  __shared__ unsigned s_last_u[kTriSlots];  // last record (stream index) copied into each slot
  __shared__ int s_tile;
  __shared__ int s_done;  // records of the current tile completed
  __shared__ int s_group;
  __shared__ double s_red[64];
  op.begin();
  bool act = op.active();
  if constexpr (CL > 1) {
    // the whole cluster follows rank 0's reading, so that all its CTAs take
    // part in the same cluster barriers (the state can only change once the
    // last tile is done, when no tile is left for anyone to take)
    if (cluster_rank() == 0 && threadIdx.x == 0) s_group = act ? 1 : 0;
    cluster_sync_all();
    act = ld_cluster_s32(cluster_map(&s_group, 0)) != 0;
    cluster_sync_all();  // s_group is reused for the group tickets
  }
  if (!act) {
    if (blockIdx.x == 0 && threadIdx.x == 0) op.inactive_end();
    return;  // no ticket touched
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool producer = wid == kTriConsumers;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kTriSlots; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
      s_last_u[s] = ~0u;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  unsigned base = 0;       // records of earlier tiles streamed by this CTA
  bool failed = false;
  while (true) {
    int k;
    TriLink<T> link;
    if constexpr (CL > 1) {
      const unsigned rank = cluster_rank();
      if (rank == 0 && threadIdx.x == 0) s_group = (int)atomicAdd(&A.ticket[0], 1u);
      cluster_sync_all();
      if (threadIdx.x == 0) s_tile = ld_cluster_s32(cluster_map(&s_group, 0));
      __syncthreads();
      const int g = s_tile;
      if ((long long)g * CL >= A.ntiles) break;  // the same for the whole cluster
      k = g * CL + (int)rank;                    // >= ntiles: idle in this group
      constexpr bool kPull = PULL;  // no room for an inbox beside the tile
      if (k < A.ntiles && rank > 0) {
        link.in0 = __ldg(A.tile_row0 + k - 1);
        link.in1 = __ldg(A.tile_row1 + k - 1);
        if constexpr (kPull) {
          link.in_remote = cluster_map(sy, rank - 1);
        } else {
          link.in = inbox;
          for (int i = threadIdx.x; i < link.in1 - link.in0; i += kTriThreads) inbox[i] = sentinel<T>();
        }
      }
      if constexpr (kPull) {
        // the successor polls this tile's array from the barrier on
        if (k < A.ntiles) {
          const int rows = __ldg(A.tile_row1 + k) - __ldg(A.tile_row0 + k);
          for (int i = threadIdx.x; i < rows; i += kTriThreads) sy[i] = sentinel<T>();
        }
      } else {
        if (k + 1 < A.ntiles && rank + 1 < (unsigned)CL) link.out = cluster_map(inbox, rank + 1);
      }
      __syncthreads();
      cluster_sync_all();  // every inbox (or pulled array) holds the sentinel before any value
    } else {
      if (threadIdx.x == 0) s_tile = (int)atomicAdd(&A.ticket[0], 1u);
      __syncthreads();
      k = s_tile;
      __syncthreads();
      if (k >= A.ntiles) break;
    }
    if (k < A.ntiles) {
      const int t0 = __ldg(A.tile_row0 + k), t1 = __ldg(A.tile_row1 + k);
      const int rec0 = __ldg(A.tile_rec + k), rec1 = __ldg(A.tile_rec + k + 1);
      const int nrec = rec1 - rec0;
      for (int q = threadIdx.x; q < nrec && q < kTriRecTable; q += kTriThreads) {
        s_roff[q] = __ldg(A.rec_off + rec0 + q);
        s_rbytes[q] = __ldg(A.rec_bytes + rec0 + q);
      }
      for (int i = threadIdx.x; i < t1 - t0; i += kTriThreads) sy[i] = sentinel<T>();
      if (threadIdx.x == 0) s_done = 0;
      __syncthreads();
      if (producer) {
        // lane j streams records j, j+L, j+2L, ... (L = kTriProdLanes): the
        // issue of a bulk copy costs about an L2 round trip, so one lane alone
        // would deliver records slower than the consumers solve them.  Slot
        // u % kTriSlots is refilled by the lane that filled it before.
        if (lane < kTriProdLanes) {
          for (int q = lane, n = 1; q < nrec && !failed; q += kTriProdLanes, ++n) {
            const unsigned u = base + q;
            const int slot = u % kTriSlots;
            if ((n & 15) == 0 && ld_volatile(A.err) != 0) {
              failed = true;
              break;
            }
            if (!mbar_wait(&empty_bar[slot], ((u / kTriSlots) & 1u) ^ 1u, A.err)) {
              failed = true;
              break;
            }
            const unsigned bytes = (unsigned)(q < kTriRecTable ? s_rbytes[q] : __ldg(A.rec_bytes + rec0 + q));
            const long long off = q < kTriRecTable ? s_roff[q] : __ldg(A.rec_off + rec0 + q);
            mbar_expect_tx(&full_bar[slot], bytes);
            tma_load_1d(ring + slot * kTriSlotBytes, A.recbuf + off, bytes, &full_bar[slot]);
            *(volatile unsigned*)&s_last_u[slot] = u;  // polled by the consumers (wait_issued)
            // after the first record is on its way: warm L2 with the vectors
            // this tile's rows read (HBM latency off the records' path)
            if (n == 1) op.prefetch(t0, t1, lane);
            // warm L2 with a record further ahead, so ring copies hit L2
            const int qa = q + kTriL2Ahead;
            if (qa < nrec && qa < kTriRecTable) tma_prefetch_l2(A.recbuf + s_roff[qa], (unsigned)s_rbytes[qa]);
          }
        }
        __syncwarp();
      } else {
        RhsAhead<OP> next;  // loads issued for this warp's next record
        for (int q = wid; q < nrec; q += kTriConsumers) {
          const unsigned u = base + q;
          const int slot = u % kTriSlots;
          const RhsAhead<OP> cur = next;
          next.have = false;
          // a lane that saw this record landed while it solved its previous
          // one (cur.have) has already waited for it
          if (!failed && !cur.have &&
              !(wait_issued(&s_last_u[slot], u, A.err) && mbar_wait(&full_bar[slot], (u / kTriSlots) & 1u, A.err)))
            failed = true;
#if GB_TRI_RHS_AHEAD
          // The next record of this warp, if it has landed: issue its
          // right-hand-side loads now, so they are in flight while this
          // record waits.  s_last_u[slot] == un means the producer has
          // issued record un into that slot (so the slot's previous record
          // was consumed and the parity test below refers to record un);
          // the barrier's phase then says whether it has landed.  Lanes
          // decide independently; a lane that sees no record loads later.
          const int qn = q + kTriConsumers;
          if (!failed && qn < nrec) {
            const unsigned un = base + qn;
            const int sn = un % kTriSlots;
            if (*(const volatile unsigned*)&s_last_u[sn] == un && mbar_try_wait(&full_bar[sn], (un / kTriSlots) & 1u)) {
              const int rn = kFixed ? record_row_fixed(ring + sn * kTriSlotBytes, lane)
                                    : record_row(ring + sn * kTriSlotBytes, lane);
              if (rn >= 0) {
                next.pr = op.pre(rn);
                next.dp = op.dpre(rn);
              }
              next.have = true;
            }
          }
#endif
          if (!failed) {
            if constexpr (kFixed)
              solve_record_fixed<POLL, OP>(A, op, sy, t0, t1, ring + slot * kTriSlotBytes, lane, &s_done, link, cur);
            else
              solve_record<T, EXACT, POLL, OP, SHORT>(A, op, sy, t0, t1, ring + slot * kTriSlotBytes, lane, &s_done,
                                                      link, cur);
          }
          __syncwarp();
          // the staged record must have been this one (its header carries its
          // index); otherwise the run stops with an error and the slot is not
          // released.  Checked off the record's path.
          if (!failed && record_index(ring + slot * kTriSlotBytes, kFixed) != rec0 + q) {
            if (lane == 0) atomicCAS(A.err, 0, (int)GB_INTERNAL);
            failed = true;
          }
          // after a failure the slot is not released: its copy may still be in
          // flight, and the producer must not aim another copy at it
          if (lane == 0 && !failed) mbar_arrive(&empty_bar[slot]);
        }
      }
      base += nrec;
      __syncthreads();
      op.chunk_end(k, A.ntiles, A.ticket, s_red);
      __syncthreads();
    }
    if constexpr (CL > 1) cluster_sync_all();  // the group's pushes are complete
  }
  // Drain: every issued copy must have landed before the CTA's shared
  // memory goes away.  A slot is refilled only after its previous record was
  // consumed, so only the last copy into each slot can still be in flight
  // (after a timeout); wait for those, bounded.  A completed copy's phase is
  // the barrier's current or immediately preceding one, so the wait on its
  // parity returns at once.
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int slot = 0; slot < kTriSlots; ++slot) {
      const unsigned u = s_last_u[slot];
      if (u == ~0u) continue;
      const uint64_t w0 = globaltimer_ns();
      while (!mbar_try_wait(&full_bar[slot], (u / kTriSlots) & 1u) &&
             globaltimer_ns() - w0 < kSpinBudgetNs) {
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
// CTAs per cluster for FP32 solves: -1 automatic (16, 8 or 4), 0 per-CTA
// form, 4, 8 or 16 forced (GBLAP_TRI_CLUSTER)
int tri_cluster_size();
// FP64 solves in pulling clusters (GBLAP_TRI_FP64_CLUSTER=0 turns them off)
bool tri_fp64_clusters();

// GB_NOT_SUPPORTED when the device cannot place one cluster of CL CTAs, or,
// with all_resident, cannot place every group's cluster at once.
template <typename T, typename OP, bool EXACT, int CL, bool PULL = false, bool POLL = false, bool SHORT = false>
int tri_launch_cl(const TriPlan& p, const TriArgs<T>& A, OP op, cudaStream_t s, size_t smem,
                  bool all_resident = false) {
  auto kern = tri_tile_kernel<T, OP, EXACT, CL, PULL, POLL, SHORT>;
  static bool attr_set = false;  // one per instantiation
  if (!attr_set) {
    GB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kTriMaxDynSmem));
    // clusters of more than 8 CTAs are an opt-in size
    if (CL > 8) GB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attr_set = true;
  }
  if constexpr (CL > 1) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(TriCons<T, SHORT>::threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const int groups = (p.ntiles + CL - 1) / CL;
    cfg.gridDim = dim3(groups * CL);
    int active = 0;
    if (cudaOccupancyMaxActiveClusters(&active, kern, &cfg) != cudaSuccess || active < 1 ||
        (all_resident && active < groups)) {
      cudaGetLastError();
      return GB_NOT_SUPPORTED;
    }
    cfg.gridDim = dim3((groups < active ? groups : active) * CL);
    GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, A, op));
    return GB_OK;
  } else {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TriCons<T, SHORT>::threads, smem) != cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
    per_sm = per_sm < tri_blocks_per_sm() ? per_sm : tri_blocks_per_sm();
    const long long cap = (long long)device_sm_count() * per_sm;
    const int grid = (int)(A.ntiles < cap ? A.ntiles : cap);
    kern<<<grid, TriCons<T, SHORT>::threads, smem, s>>>(A, op);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
}

// Launches the tiled solve: dynamic shared memory = the record ring plus one
// tile of T values (plus the inbox tile in the cluster form).  FP32 tiles
// that fit with an inbox run in clusters of 16 CTAs (8, then 4, where 16
// cannot be placed).  A tile boundary inside a cluster costs a shared-memory
// poll, one between clusters an L2 round trip; a group whose cluster is not
// resident starts only when an earlier cluster has finished all its tiles.
// On 128^3 (128 tiles, 16 of 8 or 8 of 16 groups, not all resident either
// way) 16 gave 177 ms per IC(0) split solve against 181 ms for 8.
// Everything else runs the per-CTA form on a persistent grid of
// min(tiles, SMs x resident CTAs).
template <typename T, typename OP, bool EXACT, bool POLL>
int tri_launch_form(const TriPlan& p, const TriArgs<T>& A, OP op, cudaStream_t s) {
  if (p.ntiles <= 0) return GB_OK;
  const size_t smem = (size_t)kTriSlots * kTriSlotBytes + (size_t)p.tile_rows * sizeof(T);
  if (smem > (size_t)kTriMaxDynSmem) return GB_NOT_SUPPORTED;  // an FP32-only plan in FP64
  const size_t smem_inbox = smem + (size_t)p.tile_rows * sizeof(T);
  if (sizeof(T) == 8 || smem_inbox > (size_t)kTriMaxDynSmem) {
    // clusters that pull the previous tile's values (no room for an inbox):
    // every FP64 tile, and FP32 tiles taller than half the shared memory
    const int want = tri_cluster_size();
    if (p.ntiles > 1 && !p.levels_form && want != 0 && (sizeof(T) == 4 || tri_fp64_clusters())) {
      int rc = GB_NOT_SUPPORTED;
      if (want == 16 || want < 0) rc = tri_launch_cl<T, OP, EXACT, 16, true, POLL>(p, A, op, s, smem);
      if (rc == GB_NOT_SUPPORTED && want != 16) rc = tri_launch_cl<T, OP, EXACT, 8, true, POLL>(p, A, op, s, smem);
      if (rc != GB_NOT_SUPPORTED) return rc;
    }
  }
  if constexpr (sizeof(T) == 4) {
    const size_t smem_cl = smem_inbox;
    const int want = tri_cluster_size();
    if (p.ntiles > 1 && !p.levels_form && smem_cl <= (size_t)kTriMaxDynSmem && want != 0) {
      int rc = GB_NOT_SUPPORTED;
      if (want == 16) rc = tri_launch_cl<T, OP, EXACT, 16, false, POLL>(p, A, op, s, smem_cl);
      else if (want == 8) rc = tri_launch_cl<T, OP, EXACT, 8, false, POLL>(p, A, op, s, smem_cl);
      else if (want == 4) rc = tri_launch_cl<T, OP, EXACT, 4, false, POLL>(p, A, op, s, smem_cl);
      else {
        rc = p.ntiles > 8 ? tri_launch_cl<T, OP, EXACT, 16, false, POLL>(p, A, op, s, smem_cl) : GB_NOT_SUPPORTED;
        if (rc == GB_NOT_SUPPORTED) rc = tri_launch_cl<T, OP, EXACT, 8, false, POLL>(p, A, op, s, smem_cl);
        if (rc == GB_NOT_SUPPORTED) rc = tri_launch_cl<T, OP, EXACT, 4, false, POLL>(p, A, op, s, smem_cl);
      }
      if (rc != GB_NOT_SUPPORTED) return rc;
    }
  }
  return tri_launch_cl<T, OP, EXACT, 1, false, POLL>(p, A, op, s, smem);
}

// Lower-solve OPs poll tile values where the plan's levels hold several
// records each (A.poll); the two forms are separate instantiations, since a
// runtime switch in the record code measured slower in both.
// Plans of short records only (TriPlan::short_only) in the forms large
// ones take -- thread-block clusters of 16 (pushing into an inbox where it
// fits, else pulling) or one CTA per tile -- run the SHORT instantiation;
// GB_NOT_SUPPORTED sends every other case to the general kernel.
template <typename T, typename OP, bool EXACT, bool POLL>
int tri_launch_short(const TriPlan& p, const TriArgs<T>& A, OP op, cudaStream_t s) {
  const size_t smem = (size_t)kTriSlots * kTriSlotBytes + (size_t)p.tile_rows * sizeof(T);
  const size_t smem_inbox = smem + (size_t)p.tile_rows * sizeof(T);
  if (p.ntiles <= 0) return GB_OK;
  if (smem > (size_t)kTriMaxDynSmem) return GB_NOT_SUPPORTED;  // FP32 tiles always fit
  const int want = tri_cluster_size();
  // The FP32 instantiations read the fixed layout only, and run every plan
  // in it, in every form (one CTA per tile where no cluster form applies).
  const bool fixed = sizeof(T) == 4;
  if (fixed && !p.fixed32) return GB_NOT_SUPPORTED;
  if (p.levels_form || p.ntiles <= 8 || want == 0)
    return p.levels_form || want == 0 || fixed ? tri_launch_cl<T, OP, EXACT, 1, false, POLL, true>(p, A, op, s, smem)
                                               : GB_NOT_SUPPORTED;
  if (want != 16 && want >= 0)
    return fixed ? tri_launch_cl<T, OP, EXACT, 1, false, POLL, true>(p, A, op, s, smem) : GB_NOT_SUPPORTED;
  // FP32: clusters of 16 when every group is resident at once, else of 10
  // when that makes them all resident (two fit on most GPCs), else of 16.
  // 128^3: the 128 plane tiles of either factor run in 10s (lower 249 vs
  // 257 us in 16s; 8 / 12 measured 254 / 280).
  if constexpr (sizeof(T) == 4) {
    if (smem_inbox <= (size_t)kTriMaxDynSmem) {
      int rc = tri_launch_cl<T, OP, EXACT, 16, false, POLL, true>(p, A, op, s, smem_inbox, true);
      if (rc == GB_NOT_SUPPORTED) rc = tri_launch_cl<T, OP, EXACT, 10, false, POLL, true>(p, A, op, s, smem_inbox, true);
      if (rc == GB_NOT_SUPPORTED) rc = tri_launch_cl<T, OP, EXACT, 16, false, POLL, true>(p, A, op, s, smem_inbox);
      return rc;
    }
    int rc = tri_launch_cl<T, OP, EXACT, 16, true, POLL, true>(p, A, op, s, smem, true);
    if (rc == GB_NOT_SUPPORTED) rc = tri_launch_cl<T, OP, EXACT, 10, true, POLL, true>(p, A, op, s, smem, true);
    if (rc == GB_NOT_SUPPORTED) rc = tri_launch_cl<T, OP, EXACT, 16, true, POLL, true>(p, A, op, s, smem);
    return rc;
  }
  if (!tri_fp64_clusters()) return GB_NOT_SUPPORTED;
  // FP64 lower solves in clusters of 10: two fit on most GPCs, so the 128
  // plane tiles of a 128^3 grid are all resident (in clusters of 16 only 7
  // groups of 16 are, and the eighth starts when the first has finished):
  // 319 vs 360 us there; 8 / 9 / 12 measured 346 / 322 / 388.  FP64 upper
  // and FP32 solves measured best in clusters of 16.
  if constexpr (sizeof(T) == 8) {
    if (p.lower) return tri_launch_cl<T, OP, EXACT, 10, true, POLL, true>(p, A, op, s, smem);
    return tri_launch_cl<T, OP, EXACT, 16, true, POLL, true>(p, A, op, s, smem);
  }
  return GB_NOT_SUPPORTED;
}

template <typename T, typename OP, bool EXACT>
int tri_launch(const TriPlan& p, const TriArgs<T>& A, OP op, cudaStream_t s) {
  // split hub rows: every partial-sum slot at the sentinel before the solve
  if (p.nslots > 0) GB_TRY(fill_sentinel_dev(p.nslots, A.part, s));
  // The short-record kernel: FP64 for short-only plans; FP32 exactly for the
  // plans whose FP32 records are in the fixed layout (TriPlan::fixed32),
  // which it alone reads and which the general kernel cannot.
  const bool fixed = sizeof(T) == 4 && p.fixed32;
  const bool use_short = sizeof(T) == 4 ? p.fixed32 : p.short_only;
  if constexpr (op_polls_values<OP>::value) {
    if (A.poll) {
      if (use_short) {
        const int rc = tri_launch_short<T, OP, EXACT, true>(p, A, op, s);
        if (rc != GB_NOT_SUPPORTED || fixed) return rc;
      }
      return tri_launch_form<T, OP, EXACT, true>(p, A, op, s);
    }
  }
  if (use_short) {
    const int rc = tri_launch_short<T, OP, EXACT, false>(p, A, op, s);
    if (rc != GB_NOT_SUPPORTED || fixed) return rc;
  }
  return tri_launch_form<T, OP, EXACT, false>(p, A, op, s);
}

template <typename T>
TriArgs<T> tri_args(const TriPlan& p, T* y, int* err, bool fma_form);

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
  __device__ __forceinline__ void prefetch(int r0, int r1, int part) const {
    prefetch_rows_l2(x, r0, r1, part, kTriProdLanes);
  }
  __device__ __forceinline__ void chunk_end(int, int nchunks, unsigned* ticket, double*) {
    if (threadIdx.x == 0) chunk_finished(ticket, nchunks);
  }
};

}  // namespace gb
