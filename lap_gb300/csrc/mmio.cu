// mmio.cu -- Matrix Market coordinate file -> CSR, parsed and built on the
// device.
//
// Restates LAP's read_mm_file (io_utils.c:15-74) followed by coo_to_csr
// (io_utils.c:141-235) with the same result, bit for bit:
//   * entries are "row col value" lines (1-based), values 1.0 for a
//     'pattern' file; '%' lines and blank lines are skipped;
//   * a 'symmetric' file's off-diagonal entries are mirrored;
//   * each row's entries are sorted by column, equal columns (duplicates)
//     keeping file order -- mirrored entries at the position of the line
//     that produced them -- as the reference's per-row sort of its
//     row-bucketed list does for the files it is given.
// The host reads the header; reader threads read the rest of the file in
// chunks through pinned staging, each copied to the device while the next is
// read (bytes already in host memory are copied at once).  On the device the
// whole conversion is integer and byte work bound by HBM:
//   1. newline count per 4 KB chunk, scan, line starts;
//   2. one thread per line: two integers and a decimal value, rounded to the
//      nearest double exactly (below);
//   3. a scan of valid lines gives each entry its index in the file;
//   4. keys (row, col) and values are laid out in file order, mirror beside
//      each entry, and sorted by a stable LSD radix sort (8-bit digits);
//   5. row pointers by binary search over the sorted keys.
//
// Decimal -> double.  A value with at most 19 significant digits w and a
// decimal exponent |E| <= 27 is rounded exactly with integer arithmetic:
// E >= 0: w * 5^E (< 2^127) times 2^E; E < 0: floor(w * 2^s / 5^-E) with the
// remainder as sticky bit, s chosen so the quotient has 55-56 bits, times
// 2^(-s+E).  Rounding is to nearest, ties to even, as strtod does.  Any other
// value (more digits, larger exponents, inf, nan, hex) is parsed by strtod
// on the host, for the lines that need it, packed on the device and copied
// back.
#include <cuda_runtime.h>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gb_common.cuh"
#include "gblap.h"
#include "kernels.h"

namespace gb {
namespace {

using u64 = unsigned long long;
using u128 = unsigned __int128;

constexpr int kMmThreads = 256;
constexpr int kChunkBytes = 4096;  // newline kernels: 256 threads x 16 bytes
constexpr int kScanItems = 8;      // scan: items per thread
constexpr int kScanTile = kMmThreads * kScanItems;

// line flags
enum : int { LINE_SKIP = 0, LINE_OK = 1, LINE_HOST = 2, LINE_BAD = 3 };

// ------------------------------------------------------------ scans
// Exclusive scan of n ints (total < 2^31) in three launches: tile sums, a
// single-block scan of the tile sums, tile scans plus their offsets.
__device__ __forceinline__ int block_exclusive_scan(int v, int* sm, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < kMmThreads / 32 ? sm[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kMmThreads / 32) sm[lane] = w;
  }
  __syncthreads();
  const int before = (wid ? sm[wid - 1] : 0) + x - v;
  if (total) *total = sm[kMmThreads / 32 - 1];
  __syncthreads();  // sm reused by the caller's next scan
  return before;
}

__global__ void __launch_bounds__(kMmThreads) scan_tile_sums(const int* __restrict__ in, int n, int* sums) {
  __shared__ int sm[kMmThreads / 32];
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) v += in[base + k];
  int total;
  block_exclusive_scan(v, sm, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums in place; total to *total
__global__ void __launch_bounds__(kMmThreads) scan_sums(int* sums, int nt, int* total) {
  __shared__ int sm[kMmThreads / 32];
  int carry = 0;
  for (int t0 = 0; t0 < nt; t0 += kMmThreads) {
    const int i = t0 + threadIdx.x;
    const int v = i < nt ? sums[i] : 0;
    int tot;
    const int ex = block_exclusive_scan(v, sm, &tot);
    if (i < nt) sums[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kMmThreads)
    scan_apply(const int* __restrict__ in, int n, const int* __restrict__ sums, int* out) {
  __shared__ int sm[kMmThreads / 32];
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  int run = sums[blockIdx.x] + block_exclusive_scan(s, sm, nullptr);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

// ------------------------------------------------------------ lines
__device__ __forceinline__ int count_nl16(uint4 q) {
  int c = 0;
  const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    // bytes equal to '\n' (0x0A): zero bytes of w ^ 0x0A0A0A0A
    const unsigned x = w[k] ^ 0x0A0A0A0Au;
    const unsigned z = ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x | 0x7F7F7F7Fu);
    c += __popc(z);
  }
  return c;
}

// buf holds len bytes followed by 16 zero bytes of padding (so whole
// 16-byte loads stay in the allocation); bytes at or past len never count.
__device__ __forceinline__ uint4 load16(const unsigned char* buf, long long len, long long at) {
  uint4 q = *reinterpret_cast<const uint4*>(buf + at);
  if (at + 16 > len) {  // the tail: clear bytes at or past len
    unsigned char b[16];
    memcpy(b, &q, 16);
    for (int k = 0; k < 16; ++k)
      if (at + k >= len) b[k] = 0;
    memcpy(&q, b, 16);
  }
  return q;
}

__global__ void __launch_bounds__(kMmThreads)
    nl_count_kernel(const unsigned char* __restrict__ buf, long long len, int* cnt) {
  __shared__ int sm[kMmThreads / 32];
  const long long at = (long long)blockIdx.x * kChunkBytes + threadIdx.x * 16;
  const int c = at < len ? count_nl16(load16(buf, len, at)) : 0;
  int total;
  block_exclusive_scan(c, sm, &total);
  if (threadIdx.x == 0) cnt[blockIdx.x] = total;
}

// line k + 1 starts after the k-th newline; line 0 starts at 0
__global__ void __launch_bounds__(kMmThreads)
    nl_index_kernel(const unsigned char* __restrict__ buf, long long len, const int* __restrict__ base,
                    long long* line_start) {
  __shared__ int sm[kMmThreads / 32];
  const long long at = (long long)blockIdx.x * kChunkBytes + threadIdx.x * 16;
  uint4 q = make_uint4(0, 0, 0, 0);
  if (at < len) q = load16(buf, len, at);
  int k = base[blockIdx.x] + block_exclusive_scan(at < len ? count_nl16(q) : 0, sm, nullptr);
  unsigned char b[16];
  memcpy(b, &q, 16);
#pragma unroll
  for (int j = 0; j < 16; ++j)
    if (b[j] == '\n') line_start[1 + k++] = at + j + 1;
  if (blockIdx.x == 0 && threadIdx.x == 0) line_start[0] = 0;
}

// ------------------------------------------------------------ number parsing
__device__ __forceinline__ bool is_space(unsigned char c) { return c == ' ' || c == '\t' || c == '\r'; }
__device__ __forceinline__ bool is_digit(unsigned char c) { return c >= '0' && c <= '9'; }

// unsigned decimal integer (sscanf %d accepts a sign: '+' kept, '-' is
// reported as bad, since no index may be negative)
__device__ __forceinline__ bool parse_index(const unsigned char* p, const unsigned char* end,
                                            const unsigned char** next, long long* v) {
  while (p < end && is_space(*p)) ++p;
  if (p < end && *p == '+') ++p;
  if (p >= end || !is_digit(*p)) return false;
  long long x = 0;
  while (p < end && is_digit(*p)) {
    x = x * 10 + (*p - '0');
    if (x > 0x7fffffffLL) return false;
    ++p;
  }
  *next = p;
  *v = x;
  return true;
}

__device__ __forceinline__ int msb128(u128 x) {
  const u64 hi = (u64)(x >> 64);
  return hi ? 127 - __clzll(hi) : 63 - __clzll((u64)x);
}

// m * 2^e2 rounded to the nearest double (ties to even); q > 0, and when
// sticky is set (a nonzero fraction below q's last bit) q has >= 55 bits.
__device__ __forceinline__ double make_double(u128 q, int e2, bool sticky, bool neg) {
  const int p = msb128(q);
  u64 m;
  int ex;
  if (p <= 52) {
    m = (u64)q << (52 - p);
    ex = e2 - (52 - p);
  } else {
    int sh = p - 52;
    m = (u64)(q >> sh);
    const u128 rem = q & (((u128)1 << sh) - 1);
    const u128 half = (u128)1 << (sh - 1);
    const bool up = rem > half || (rem == half && (sticky || (m & 1)));
    if (up && ++m == (1ULL << 53)) {
      m >>= 1;
      ++sh;
    }
    ex = e2 + sh;
  }
  const u64 bits = ((u64)(neg ? 1 : 0) << 63) | ((u64)(ex + 52 + 1023) << 52) | (m & ((1ULL << 52) - 1));
  return __longlong_as_double((long long)bits);
}

// floor((hi * 2^64 + lo) / d) and the remainder, for hi < d (quotient < 2^64)
__device__ __forceinline__ u64 div128by64(u64 hi, u64 lo, u64 d, u64* r) {
  u64 q = 0, x = hi;
  for (int i = 63; i >= 0; --i) {
    const bool carry = x >> 63;
    x = (x << 1) | ((lo >> i) & 1);
    if (carry || x >= d) {
      x -= d;
      q |= 1ULL << i;
    }
  }
  *r = x;
  return q;
}

__device__ __forceinline__ u64 pow5(int k) {  // k <= 27: 5^27 < 2^63
  u64 p = 1;
  for (int i = 0; i < k; ++i) p *= 5;
  return p;
}

// Decimal value [+-]digits[.digits][(e|E)[+-]digits]: 0 = parsed, 1 =
// outside the exact path (the host parses it), -1 = not a number.
__device__ int parse_real(const unsigned char* p, const unsigned char* end, double* v) {
  while (p < end && is_space(*p)) ++p;
  bool neg = false;
  if (p < end && (*p == '+' || *p == '-')) neg = *p++ == '-';
  u64 w = 0;
  int nd = 0, dexp = 0;
  bool any = false, many = false;
  while (p < end && is_digit(*p)) {
    any = true;
    if (nd < 19) {
      if (w || *p != '0') {
        w = w * 10 + (*p - '0');
        ++nd;
      }
    } else {
      many = true;
      ++dexp;  // a dropped integer digit still scales the value
    }
    ++p;
  }
  if (p < end && *p == '.') {
    ++p;
    while (p < end && is_digit(*p)) {
      any = true;
      if (nd < 19) {
        if (w || *p != '0') {
          w = w * 10 + (*p - '0');
          ++nd;
        }
        --dexp;
      } else {
        many = true;
      }
      ++p;
    }
  }
  if (!any) {
    // inf, nan, hex and the like: the host decides
    return (p < end && !is_space(*p) && *p != '\n') ? 1 : -1;
  }
  int e = 0;
  if (p < end && (*p == 'e' || *p == 'E')) {
    const unsigned char* q = p + 1;
    bool eneg = false;
    if (q < end && (*q == '+' || *q == '-')) eneg = *q++ == '-';
    if (q < end && is_digit(*q)) {
      while (q < end && is_digit(*q)) {
        if (e < 100000) e = e * 10 + (*q - '0');
        ++q;
      }
      if (eneg) e = -e;
      p = q;
    }
  }
  if (p < end && !is_space(*p) && *p != '\n') return 1;  // trailing characters: as strtod would see them
  if (many) return 1;
  if (w == 0) {
    *v = neg ? -0.0 : 0.0;
    return 0;
  }
  int E = dexp + e;
  while (E < -27 && w % 10 == 0) {  // trailing zeros of the digits
    w /= 10;
    ++E;
  }
  if (E > 27 || E < -27) return 1;
  if (E >= 0) {
    const u64 f = pow5(E);
    const u128 N = (u128)w * f;
    *v = make_double(N, E, false, neg);
    return 0;
  }
  const int k = -E;
  const u64 d = pow5(k);
  const int bw = 64 - __clzll(w), bd = 64 - __clzll(d);
  const int s = max(0, 55 + bd - bw);  // quotient >= 2^54, dividend < 2^118
  const u128 X = (u128)w << s;
  u64 r;
  const u64 q = div128by64((u64)(X >> 64), (u64)X, d, &r);
  *v = make_double((u128)q, -s - k, r != 0, neg);
  return 0;
}

// One thread per line: flag, row, column and value of the line's entry.
__global__ void __launch_bounds__(kMmThreads)
    parse_lines_kernel(const unsigned char* __restrict__ buf, const long long* __restrict__ line_start, int L,
                       int n, int m, int pattern, int* flag, int* row, int* col, double* val, int* host_lines,
                       int* nhost, int* nbad) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  const unsigned char* p = buf + line_start[l];
  const unsigned char* end = buf + line_start[l + 1];
  while (p < end && is_space(*p)) ++p;
  int f = LINE_SKIP;
  if (p < end && *p != '%' && *p != '\n') {
    long long r = 0, c = 0;
    const unsigned char* q = p;
    f = LINE_BAD;
    if (parse_index(q, end, &q, &r) && parse_index(q, end, &q, &c) && r >= 1 && r <= n && c >= 1 && c <= m) {
      double v = 1.0;
      int pr = 0;
      if (!pattern) pr = parse_real(q, end, &v);
      if (pr == 0) f = LINE_OK;
      else if (pr == 1) f = LINE_HOST;
      row[l] = (int)r - 1;
      col[l] = (int)c - 1;
      val[l] = v;
    }
  }
  if (f == LINE_HOST) host_lines[atomicAdd(nhost, 1)] = l;
  if (f == LINE_BAD) atomicAdd(nbad, 1);
  flag[l] = f != LINE_SKIP && f != LINE_BAD ? 1 : 0;
}

// start and end of each line the host parses
__global__ void gather_lines_kernel(int k, const int* __restrict__ lines, const long long* __restrict__ ls,
                                    long long* se) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) {
    se[2 * i] = ls[lines[i]];
    se[2 * i + 1] = ls[lines[i] + 1];
  }
}

// the bytes of those lines, packed end to end for one copy to the host
// (one block per line; se and po hold offsets inside buf and out)
__global__ void pack_lines_kernel(int k, const long long* __restrict__ se, const long long* __restrict__ po,
                                  const unsigned char* __restrict__ buf, char* __restrict__ out) {
  const int i = blockIdx.x;
  if (i >= k) return;
  const long long s0 = se[2 * i], len = se[2 * i + 1] - s0, o = po[i];
  for (long long j = threadIdx.x; j < len; j += blockDim.x) out[o + j] = (char)buf[s0 + j];
}

// host-parsed values into their lines
__global__ void patch_values_kernel(int k, const int* __restrict__ lines, const double* __restrict__ v, double* val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) val[lines[i]] = v[i];
}

// ------------------------------------------------------------ keys
// Entry e (the rank of its line among valid lines, e < nnz) goes to slot
// e (general) or 2e, its mirror to 2e + 1 (symmetric; the sentinel row n
// when it is a diagonal entry).  Keys are row << cb | col.
__global__ void __launch_bounds__(kMmThreads)
    make_keys_kernel(int L, const int* __restrict__ flag, const int* __restrict__ rank, const int* __restrict__ row,
                     const int* __restrict__ col, const double* __restrict__ val, long long nnz, int symmetric,
                     int cb, int n, u64* keys, double* vals, int* ndiag) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L || !flag[l]) return;
  const long long e = rank[l];
  if (e >= nnz) return;  // lines past the header's count are ignored
  const u64 r = (u64)row[l], c = (u64)col[l];
  const double v = val[l];
  if (!symmetric) {
    keys[e] = r << cb | c;
    vals[e] = v;
    return;
  }
  keys[2 * e] = r << cb | c;
  vals[2 * e] = v;
  if (r != c) {
    keys[2 * e + 1] = c << cb | r;
    vals[2 * e + 1] = v;
  } else {
    keys[2 * e + 1] = (u64)n << cb;
    vals[2 * e + 1] = 0.0;
    atomicAdd(ndiag, 1);
  }
}

// Adjacency files (read_adjacency_file, io_utils.c:128-135): after the file's
// entries, one unit diagonal entry per vertex, entry index nnz + j.
__global__ void diag_keys_kernel(int n, long long nnz, int cb, u64* keys, double* vals, int* ndiag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const long long e = nnz + j;
  keys[2 * e] = (u64)j << cb | (u64)j;
  vals[2 * e] = 1.0;
  keys[2 * e + 1] = (u64)n << cb;
  vals[2 * e + 1] = 0.0;
  atomicAdd(ndiag, 1);
}

// ------------------------------------------------------------ radix sort
// Stable LSD radix sort of (key, value) pairs, 8-bit digits.  A block takes
// a tile of 16 items per thread; warp w owns items [w * 512, (w + 1) * 512)
// of the tile, 32 at a time, so ranks follow item order.
constexpr int kRsItems = 16;
constexpr int kRsTile = kMmThreads * kRsItems;
constexpr int kRsWarps = kMmThreads / 32;

__global__ void __launch_bounds__(kMmThreads)
    rs_hist_kernel(const u64* __restrict__ keys, long long n, int shift, int* hist) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kRsTile;
#pragma unroll 4
  for (int k = 0; k < kRsItems; ++k) {
    const long long i = base + k * kMmThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(int)((keys[i] >> shift) & 255)], 1);
  }
  __syncthreads();
  hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];  // digit-major for the scan
}

__global__ void __launch_bounds__(kMmThreads)
    rs_scatter_kernel(const u64* __restrict__ kin, const double* __restrict__ vin, u64* __restrict__ kout,
                      double* __restrict__ vout, long long n, int shift, const int* __restrict__ offs) {
  __shared__ int wc[kRsWarps][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = threadIdx.x; t < kRsWarps * 256; t += kMmThreads) wc[t / 256][t % 256] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kRsTile + (long long)w * (kRsItems * 32);
  const unsigned lt = (1u << lane) - 1u;
  int pos[kRsItems];
#pragma unroll
  for (int k = 0; k < kRsItems; ++k) {
    const long long i = base + k * 32 + lane;
    const int d = i < n ? (int)((kin[i] >> shift) & 255) : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int before = d < 256 ? wc[w][d] : 0;
    pos[k] = before + __popc(peers & lt);
    __syncwarp();
    if (d < 256 && (peers & lt) == 0) wc[w][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: exclusive offsets of the warps
  {
    const int d = threadIdx.x;
    int run = 0;
    for (int ww = 0; ww < kRsWarps; ++ww) {
      const int c = wc[ww][d];
      wc[ww][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kRsItems; ++k) {
    const long long i = base + k * 32 + lane;
    if (i < n) {
      const u64 key = kin[i];
      const int d = (int)((key >> shift) & 255);
      const long long dst = (long long)offs[d * gridDim.x + blockIdx.x] + wc[w][d] + pos[k];
      kout[dst] = key;
      vout[dst] = vin[i];
    }
  }
}

// ------------------------------------------------------------ CSR
// ia[r] = number of keys with row < r (binary search over the sorted keys)
__global__ void row_ptr_kernel(const u64* __restrict__ keys, long long nk, int n, int cb, int* ia) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > n) return;
  long long lo = 0, hi = nk;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if ((long long)(keys[mid] >> cb) < r) lo = mid + 1;
    else hi = mid;
  }
  ia[r] = (int)lo;
}

__global__ void cols_vals_kernel(const u64* __restrict__ keys, const double* __restrict__ vals, long long nk,
                                 u64 cmask, int* ja, double* a) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += (long long)gridDim.x * blockDim.x) {
    ja[k] = (int)(keys[k] & cmask);
    a[k] = vals[k];
  }
}

// ------------------------------------------------------------ Laplacian
// create_L_and_split (io_utils.c:367-491) on A's CSR in place.  Degrees:
// DD[i] = -1 plus the row's values, summed left to right into an int, so
// every partial sum is truncated toward zero (io_utils.c:387-395); exact = 1
// sums in double instead.  One thread per row keeps that order.
__global__ void lap_degree_kernel(int n, const int* __restrict__ ia, const double* __restrict__ a, int exact,
                                  double* deg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (exact) {
    double d = -1.0;
    for (int k = ia[i]; k < ia[i + 1]; ++k) d += a[k];
    deg[i] = d;
  } else {
    int d = -1;
    for (int k = ia[i]; k < ia[i + 1]; ++k) d = (int)((double)d + a[k]);
    deg[i] = (double)d;
  }
}

// unweighted: diagonal = degree, off-diagonal = -w; weighted: diagonal 1,
// off-diagonal ((-1 * w) * (1/sqrt(d_i))) * (1/sqrt(d_j)), in the
// reference's order of operations
__global__ void lap_values_kernel(int n, const int* __restrict__ ia, const int* __restrict__ ja, double* a,
                                  const double* __restrict__ deg, int weighted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dsq = weighted ? 1.0 / sqrt(deg[i]) : 0.0;
  for (int k = ia[i]; k < ia[i + 1]; ++k) {
    const int c = ja[k];
    if (c == i) a[k] = weighted ? 1.0 : deg[i];
    else if (!weighted) a[k] = (-1.0) * a[k];
    else a[k] = __dmul_rn(__dmul_rn((-1.0) * a[k], dsq), 1.0 / sqrt(deg[c]));
  }
}

// ------------------------------------------------------------ host
// What to build from the file.
struct MmMode {
  bool adjacency = false;  // read_adjacency_file: symmetric, unit diagonal placeholders
  bool laplacian = false;  // then create_L_and_split's in-place Laplacian
  int weighted = 0, exact = 0;
};

struct Header {
  bool pattern = false, symmetric = false;
  long long n = 0, m = 0, nnz = 0;
  long long data_off = 0;  // first byte after the size line
};

// The banner, '%' comment lines and the size line (io_utils.c:24-44).
bool parse_header(const char* b, long long len, Header* h) {
  long long p = 0;
  auto line_end = [&](long long at) {
    while (at < len && b[at] != '\n') ++at;
    return at;
  };
  long long e = line_end(0);
  const std::string banner(b, (size_t)e);
  h->pattern = banner.find("pattern") != std::string::npos;
  h->symmetric = banner.find("symmetric") != std::string::npos;
  p = e + 1;
  // the banner line itself starts with '%'; skip further comment lines
  while (p < len && b[p] == '%') p = line_end(p) + 1;
  if (p >= len) return false;
  e = line_end(p);
  const std::string size_line(b + p, (size_t)(e - p));
  if (sscanf(size_line.c_str(), "%lld %lld %lld", &h->n, &h->m, &h->nnz) != 3) return false;
  h->data_off = std::min(len, e + 1);
  return true;
}

struct DevBufs {
  std::vector<void*> v;
  template <typename T>
  int get(T** p, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
      cudaGetLastError();
      return GB_NO_MEMORY;
    }
    v.push_back(q);
    *p = static_cast<T*>(q);
    return GB_OK;
  }
  ~DevBufs() {
    for (void* q : v) cudaFree(q);
  }
};

int scan_exclusive(DevBufs& D, const int* in, int n, int* out, int* total_dev, cudaStream_t s) {
  const int nt = std::max(1, ceil_div(n, kScanTile));
  int* sums = nullptr;
  GB_TRY(D.get(&sums, nt));
  scan_tile_sums<<<nt, kMmThreads, 0, s>>>(in, n, sums);
  scan_sums<<<1, kMmThreads, 0, s>>>(sums, nt, total_dev);
  scan_apply<<<nt, kMmThreads, 0, s>>>(in, n, sums, out);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int bits_for(long long v) {  // bits to hold 0..v
  int b = 1;
  while (b < 62 && (1LL << b) <= v) ++b;
  return b;
}

// Reader threads and the pinned staging they share: each thread owns two
// chunks of staging and alternates between them, reading one while the
// other's copy to the device is in flight.
constexpr long long kReadChunk = 4ll << 20;
constexpr int kReadThreadsMax = 8;

int read_threads() {
  int t = kReadThreadsMax;
  if (const char* e = getenv("GBLAP_MM_READ_THREADS")) t = atoi(e);
  const int hw = (int)std::thread::hardware_concurrency();
  if (hw > 0) t = std::min(t, hw);
  return std::max(1, std::min(t, kReadThreadsMax));
}

// Pinned staging kept for the process's lifetime (like the CUDA context it
// belongs to): pinning the whole file, or even 64 MB, per call costs more
// than reading it.  One reader at a time holds it.
struct Staging {
  std::mutex mu;
  unsigned char* p = nullptr;
  size_t bytes = 0;
};
Staging& staging() {
  static Staging* st = new Staging();
  return *st;
}

// Bytes [off, off + n) of the open file into device memory dst.  Chunk c
// goes to thread c % T, which preads it into its free staging chunk and
// copies it to the device on its own stream while reading its next chunk,
// so the page-cache copy runs on T cores and overlaps the transfer.
// Returns after every copy has completed.
int read_file_to_device(int fd, long long off, long long n, unsigned char* dst) {
  if (n <= 0) return GB_OK;
  const long long nch = (n + kReadChunk - 1) / kReadChunk;
  const int T = (int)std::min<long long>(nch, read_threads());
  Staging& st = staging();
  std::lock_guard<std::mutex> lock(st.mu);
  const size_t need = (size_t)2 * kReadThreadsMax * kReadChunk;
  if (st.bytes < need) {
    if (st.p) cudaFreeHost(st.p);
    st.p = nullptr;
    st.bytes = 0;
    if (cudaMallocHost(&st.p, need) != cudaSuccess) {
      cudaGetLastError();
      st.p = nullptr;
      return GB_NO_MEMORY;
    }
    st.bytes = need;
  }
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  std::atomic<int> err{GB_OK};
  auto fail = [&](int code) {
    int ok = GB_OK;
    err.compare_exchange_strong(ok, code);
  };
  auto work = [&](int t) {
    cudaStream_t cs = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (cudaSetDevice(dev) != cudaSuccess || cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      fail(GB_CUDA_ERROR);
    } else {
      int j = 0;
      for (long long c = t; c < nch && err.load() == GB_OK; c += T, ++j) {
        unsigned char* sb = st.p + (size_t)(2 * t + (j & 1)) * kReadChunk;
        // the chunk's earlier copy out of this staging must have left it
        if (j >= 2 && cudaEventSynchronize(ev[j & 1]) != cudaSuccess) {
          fail(GB_CUDA_ERROR);
          break;
        }
        const long long o = c * kReadChunk, m = std::min(kReadChunk, n - o);
        long long got = 0;
        while (got < m) {
          const ssize_t r = pread(fd, sb + got, (size_t)(m - got), (off_t)(off + o + got));
          if (r < 0 && errno == EINTR) continue;
          if (r <= 0) break;
          got += r;
        }
        if (got < m) {
          fail(GB_BAD_INPUT);
          break;
        }
        if (cudaMemcpyAsync(dst + o, sb, (size_t)m, cudaMemcpyHostToDevice, cs) != cudaSuccess ||
            cudaEventRecord(ev[j & 1], cs) != cudaSuccess) {
          fail(GB_CUDA_ERROR);
          break;
        }
      }
    }
    if (cs && cudaStreamSynchronize(cs) != cudaSuccess) fail(GB_CUDA_ERROR);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (cs) cudaStreamDestroy(cs);
  };
  std::vector<std::thread> th;
  for (int t = 1; t < T; ++t) {
    try {
      th.emplace_back(work, t);
    } catch (...) {  // no thread: its chunks stay unread, so the read fails as a whole
      fail(GB_NO_MEMORY);
      break;
    }
  }
  work(0);
  for (auto& x : th) x.join();
  if (err.load() == GB_BAD_INPUT) fprintf(stderr, "libgblap: Matrix Market: short read\n");
  return err.load();
}

// Where the bytes after the size line come from: the whole input in host
// memory, or an open file read by read_file_to_device.
struct MmSource {
  const char* hb = nullptr;
  int fd = -1;
};

int mm_csr_build(Header h, long long len, const MmSource& src, gb_mm_csr* out, double read_ms, const MmMode& mode);

// The conversion from host bytes (the whole file).
int mm_csr_from_bytes(const char* hb, long long len, gb_mm_csr* out, double read_ms, const MmMode& mode) {
  Header h;
  if (!parse_header(hb, len, &h)) {
    fprintf(stderr, "libgblap: Matrix Market: no size line\n");
    return GB_BAD_INPUT;
  }
  MmSource src;
  src.hb = hb;
  return mm_csr_build(h, len, src, out, read_ms, mode);
}

int mm_csr_build(Header h, long long len, const MmSource& src, gb_mm_csr* out, double read_ms, const MmMode& mode) {
  if (mode.adjacency) h.symmetric = true;  // io_utils.c:96
  if (h.n <= 0 || h.m <= 0 || h.nnz < 0 || h.n >= (1LL << 31) - 1 || h.m >= (1LL << 31) - 1 ||
      (h.symmetric ? 2 : 1) * h.nnz >= (1LL << 31) - 1)
    return h.n <= 0 || h.m <= 0 || h.nnz < 0 ? GB_BAD_INPUT : GB_NOT_SUPPORTED;
  const long long dlen = len - h.data_off;
  const int n = (int)h.n, m = (int)h.m;
  cudaStream_t s;
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DevBufs D;  // freed after the stream guard below has synchronised
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  } sg{s};
  cudaEvent_t ev[3];
  for (auto& e : ev) GB_CUDA_TRY(cudaEventCreate(&e));
  struct EventGuard {
    cudaEvent_t* e;
    ~EventGuard() {
      for (int i = 0; i < 3; ++i) cudaEventDestroy(e[i]);
    }
  } eg{ev};
  // bytes, padded to whole 16-byte loads
  unsigned char* buf = nullptr;
  GB_TRY(D.get(&buf, (size_t)dlen + 32));
  if (src.fd >= 0 && dlen > 0) {  // a file: read and copied in overlapped chunks, counted as the read
    const auto t0 = std::chrono::steady_clock::now();
    GB_TRY(read_file_to_device(src.fd, h.data_off, dlen, buf));
    read_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  GB_CUDA_TRY(cudaEventRecord(ev[0], s));
  GB_CUDA_TRY(cudaMemsetAsync(buf + dlen, 0, 32, s));
  if (src.hb && dlen > 0)
    GB_CUDA_TRY(cudaMemcpyAsync(buf, src.hb + h.data_off, (size_t)dlen, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaEventRecord(ev[1], s));
  // 1. lines
  const int nchunk = (int)std::max(1LL, (dlen + kChunkBytes - 1) / kChunkBytes);
  int *nlc = nullptr, *nlb = nullptr, *ctl = nullptr;
  GB_TRY(D.get(&nlc, nchunk));
  GB_TRY(D.get(&nlb, nchunk));
  GB_TRY(D.get(&ctl, 8));  // [0] newlines, [1] host lines, [2] bad lines, [3] valid lines, [4] diagonal mirrors
  GB_CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(int) * 8, s));
  nl_count_kernel<<<nchunk, kMmThreads, 0, s>>>(buf, dlen, nlc);
  GB_TRY(scan_exclusive(D, nlc, nchunk, nlb, ctl + 0, s));
  int nl = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&nl, ctl + 0, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  const int L = nl + 1;  // the last line may be empty
  long long* ls = nullptr;
  GB_TRY(D.get(&ls, (size_t)L + 1));
  nl_index_kernel<<<nchunk, kMmThreads, 0, s>>>(buf, dlen, nlb, ls);
  GB_CUDA_TRY(cudaMemcpyAsync(ls + L, &dlen, sizeof(long long), cudaMemcpyHostToDevice, s));
  // 2. parse
  int *flag = nullptr, *row = nullptr, *col = nullptr, *rank = nullptr, *hl = nullptr;
  double* val = nullptr;
  GB_TRY(D.get(&flag, L));
  GB_TRY(D.get(&row, L));
  GB_TRY(D.get(&col, L));
  GB_TRY(D.get(&rank, L));
  GB_TRY(D.get(&hl, L));
  GB_TRY(D.get(&val, L));
  parse_lines_kernel<<<ceil_div(L, kMmThreads), kMmThreads, 0, s>>>(buf, ls, L, n, m, h.pattern ? 1 : 0, flag, row,
                                                                      col, val, hl, ctl + 1, ctl + 2);
  GB_CUDA_TRY(cudaGetLastError());
  // 3. entry index of each valid line
  GB_TRY(scan_exclusive(D, flag, L, rank, ctl + 3, s));
  int hc[8];
  GB_CUDA_TRY(cudaMemcpyAsync(hc, ctl, sizeof hc, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (hc[2] > 0) {
    fprintf(stderr, "libgblap: Matrix Market: %d malformed or out-of-range entries\n", hc[2]);
    return GB_BAD_INPUT;
  }
  if (hc[3] < h.nnz) {
    fprintf(stderr, "libgblap: Matrix Market file ended after %d of %lld entries\n", hc[3], h.nnz);
    return GB_BAD_INPUT;
  }
  // values the exact path left to strtod
  const int nh = hc[1];
  if (nh > 0) {
    long long* dse = nullptr;
    double* dv = nullptr;
    GB_TRY(D.get(&dse, 2 * (size_t)nh));
    GB_TRY(D.get(&dv, nh));
    gather_lines_kernel<<<ceil_div(nh, 256), 256, 0, s>>>(nh, hl, ls, dse);
    std::vector<long long> se(2 * (size_t)nh);
    GB_CUDA_TRY(cudaMemcpyAsync(se.data(), dse, sizeof(long long) * 2 * nh, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    // the lines' bytes from the device copy (a file's bytes are not kept on the host)
    std::vector<long long> po(nh + 1, 0);
    for (int i = 0; i < nh; ++i) po[i + 1] = po[i] + (se[2 * i + 1] - se[2 * i]);
    long long* dpo = nullptr;
    char* dpk = nullptr;
    GB_TRY(D.get(&dpo, nh));
    GB_TRY(D.get(&dpk, (size_t)po[nh]));
    GB_CUDA_TRY(cudaMemcpyAsync(dpo, po.data(), sizeof(long long) * nh, cudaMemcpyHostToDevice, s));
    pack_lines_kernel<<<nh, 128, 0, s>>>(nh, dse, dpo, buf, dpk);
    std::vector<char> pk((size_t)po[nh] + 1);
    if (po[nh] > 0) GB_CUDA_TRY(cudaMemcpyAsync(pk.data(), dpk, (size_t)po[nh], cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<double> vals(nh);
    for (int i = 0; i < nh; ++i) {
      const std::string line(pk.data() + po[i], (size_t)(po[i + 1] - po[i]));
      long long r, c;
      double v = 0.0;
      sscanf(line.c_str(), "%lld %lld %lf", &r, &c, &v);
      vals[i] = v;
    }
    GB_CUDA_TRY(cudaMemcpyAsync(dv, vals.data(), sizeof(double) * nh, cudaMemcpyHostToDevice, s));
    patch_values_kernel<<<ceil_div(nh, 256), 256, 0, s>>>(nh, hl, dv, val);
    GB_CUDA_TRY(cudaStreamSynchronize(s));
  }
  // 4. keys in file order, then the sort
  const long long entries = h.nnz + (mode.adjacency ? h.n : 0);
  if ((h.symmetric ? 2 : 1) * entries >= (1LL << 31) - 1) return GB_NOT_SUPPORTED;
  const long long slots = (h.symmetric ? 2 : 1) * entries;
  const int cb = bits_for(std::max(m - 1, 1));
  const int rb = bits_for(n);  // row n is the sentinel
  u64 *k0 = nullptr, *k1 = nullptr;
  double *v0 = nullptr, *v1 = nullptr;
  GB_TRY(D.get(&k0, slots));
  GB_TRY(D.get(&k1, slots));
  GB_TRY(D.get(&v0, slots));
  GB_TRY(D.get(&v1, slots));
  make_keys_kernel<<<ceil_div(L, kMmThreads), kMmThreads, 0, s>>>(L, flag, rank, row, col, val, h.nnz,
                                                                   h.symmetric ? 1 : 0, cb, n, k0, v0, ctl + 4);
  if (mode.adjacency) diag_keys_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, h.nnz, cb, k0, v0, ctl + 4);
  GB_CUDA_TRY(cudaGetLastError());
  if (slots > 0) {
    const int nblk = (int)((slots + kRsTile - 1) / kRsTile);
    int *hist = nullptr, *offs = nullptr;
    GB_TRY(D.get(&hist, (size_t)256 * nblk));
    GB_TRY(D.get(&offs, (size_t)256 * nblk));
    for (int shift = 0; shift < cb + rb; shift += 8) {
      rs_hist_kernel<<<nblk, kMmThreads, 0, s>>>(k0, slots, shift, hist);
      GB_TRY(scan_exclusive(D, hist, 256 * nblk, offs, ctl + 5, s));
      rs_scatter_kernel<<<nblk, kMmThreads, 0, s>>>(k0, v0, k1, v1, slots, shift, offs);
      GB_CUDA_TRY(cudaGetLastError());
      std::swap(k0, k1);
      std::swap(v0, v1);
    }
  }
  int ndiag = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&ndiag, ctl + 4, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  const long long nk = slots - (h.symmetric ? ndiag : 0);
  // 5. CSR (owned by the caller)
  int *ia = nullptr, *ja = nullptr;
  double* a = nullptr;
  if (cudaMalloc(&ia, sizeof(int) * ((size_t)n + 1)) != cudaSuccess ||
      cudaMalloc(&ja, sizeof(int) * std::max<size_t>((size_t)nk, 1)) != cudaSuccess ||
      cudaMalloc(&a, sizeof(double) * std::max<size_t>((size_t)nk, 1)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(ia);
    cudaFree(ja);
    cudaFree(a);
    return GB_NO_MEMORY;
  }
  row_ptr_kernel<<<ceil_div(n + 1, 256), 256, 0, s>>>(k0, nk, n, cb, ia);
  cols_vals_kernel<<<std::max(1, std::min(ceil_div((int)std::min<long long>(nk, 1 << 30), 256), 8 * device_sm_count())),
                     256, 0, s>>>(k0, v0, nk, (1ULL << cb) - 1, ja, a);
  if (mode.laplacian) {
    double* deg = nullptr;
    GB_TRY(D.get(&deg, n));
    lap_degree_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, ia, a, mode.exact, deg);
    lap_values_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, ia, ja, a, deg, mode.weighted);
  }
  GB_CUDA_TRY(cudaEventRecord(ev[2], s));
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    cudaFree(ia);
    cudaFree(ja);
    cudaFree(a);
    return GB_CUDA_ERROR;
  }
  float h2d = 0.f, dev = 0.f;
  cudaEventElapsedTime(&h2d, ev[0], ev[1]);
  cudaEventElapsedTime(&dev, ev[1], ev[2]);
  out->n = n;
  out->m = m;
  out->nnz_file = h.nnz;
  out->nnz = (int)nk;
  out->symmetric = h.symmetric ? 1 : 0;
  out->pattern = h.pattern ? 1 : 0;
  out->ia = ia;
  out->ja = ja;
  out->a = a;
  out->host_parsed = nh;
  out->read_ms = read_ms;
  out->h2d_ms = h2d;
  out->device_ms = dev;
  return GB_OK;
}

}  // namespace
}  // namespace gb

extern "C" int gb_mm_parse_csr(const char* bytes, long long len, gb_mm_csr* out) {
  if (!bytes || len <= 0 || !out) return GB_BAD_INPUT;
  memset(out, 0, sizeof *out);
  return gb::mm_csr_from_bytes(bytes, len, out, 0.0, gb::MmMode());
}

namespace gb {
namespace {
int mm_read_file(const char* path, gb_mm_csr* out, const MmMode& mode) {
  if (!path || !out) return GB_BAD_INPUT;
  memset(out, 0, sizeof *out);
  const auto t0 = std::chrono::steady_clock::now();
  const int fd = open(path, O_RDONLY);
  if (fd < 0) {
    fprintf(stderr, "libgblap: gb_mm_read_csr: cannot open %s\n", path);
    return GB_BAD_INPUT;
  }
  struct FdGuard {
    int fd;
    ~FdGuard() { close(fd); }
  } fg{fd};
  struct stat sb;
  if (fstat(fd, &sb) != 0 || sb.st_size <= 0) return GB_BAD_INPUT;
  const long long len = (long long)sb.st_size;
  // the banner, comments and size line, read until the size line ends
  // inside what was read (or the file does)
  std::vector<char> head;
  Header h;
  for (long long want = std::min(len, 1ll << 16);; want = std::min(len, 2 * want)) {
    head.resize((size_t)want);
    long long got = 0;
    while (got < want) {
      const ssize_t r = pread(fd, head.data() + got, (size_t)(want - got), (off_t)got);
      if (r < 0 && errno == EINTR) continue;
      if (r <= 0) break;
      got += r;
    }
    if (got < want) return GB_BAD_INPUT;
    const bool ok = parse_header(head.data(), want, &h);
    if (ok && (want == len || (h.data_off <= want && head[(size_t)h.data_off - 1] == '\n'))) break;
    if (want == len) {
      fprintf(stderr, "libgblap: Matrix Market: no size line\n");
      return GB_BAD_INPUT;
    }
  }
  const double head_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  MmSource src;
  src.fd = fd;
  return mm_csr_build(h, len, src, out, head_ms, mode);
}

MmMode laplacian_mode(int weighted, int exact) {
  MmMode m;
  m.adjacency = m.laplacian = true;
  m.weighted = weighted ? 1 : 0;
  m.exact = exact ? 1 : 0;
  return m;
}
}  // namespace
}  // namespace gb

extern "C" int gb_mm_read_csr(const char* path, gb_mm_csr* out) { return gb::mm_read_file(path, out, gb::MmMode()); }

extern "C" int gb_mm_read_laplacian(const char* path, int weighted, int exact_degrees, gb_mm_csr* out) {
  return gb::mm_read_file(path, out, gb::laplacian_mode(weighted, exact_degrees));
}

extern "C" int gb_mm_parse_laplacian(const char* bytes, long long len, int weighted, int exact_degrees,
                                     gb_mm_csr* out) {
  if (!bytes || len <= 0 || !out) return GB_BAD_INPUT;
  memset(out, 0, sizeof *out);
  return gb::mm_csr_from_bytes(bytes, len, out, 0.0, gb::laplacian_mode(weighted, exact_degrees));
}

extern "C" int gb_mm_csr_free(gb_mm_csr* m) {
  if (!m) return GB_BAD_INPUT;
  cudaFree(m->ia);
  cudaFree(m->ja);
  cudaFree(m->a);
  m->ia = m->ja = nullptr;
  m->a = nullptr;
  return GB_OK;
}

// ------------------------------------------------------------ projected right-hand side
// cg_driver.c:159-230: b_i = (-1)^i, then b minus its component along the
// Laplacian's null vector -- e / sqrt(n) (unweighted), or sqrt(d) e /
// ||sqrt(d) e|| (weighted, d the diagonal) -- with the same BLAS-1 calls in
// the same order (scal, dot, axpy; vector_sqrt, vec_vec), on the legacy
// default stream as LAP's backend runs them.
extern "C" double cuda_dot(const int n, const double* v, const double* w);
extern "C" void cuda_scal(const int n, const double alpha, double* v);
extern "C" void cuda_axpy(const int n, const double alpha, const double* x, double* y);
extern "C" void cuda_vec_vec(const int n, const double* x, const double* y, double* res);
extern "C" void cuda_vector_sqrt(const int n, const double* v, double* res);

namespace gb {
namespace {
__global__ void rhs_init_kernel(int n, double* b, double* e) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  b[i] = (i % 2) ? -1.0 : 1.0;  // pow(-1.0, i % 2)
  e[i] = 1.0;
}
__global__ void diagonal_kernel(int n, const int* __restrict__ ia, const int* __restrict__ ja,
                                const double* __restrict__ a, double* d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = 0.0;
  for (int k = ia[i]; k < ia[i + 1]; ++k)
    if (ja[k] == i) v = a[k];
  d[i] = v;
}
}  // namespace
}  // namespace gb

extern "C" int gb_laplacian_rhs(int n, const int* ia, const int* ja, const double* a, int weighted, double* b,
                                double* work) {
  if (n <= 0 || !b || !work || (weighted && (!ia || !ja || !a))) return GB_BAD_INPUT;
  double* e = work;  // [n]
  gb::rhs_init_kernel<<<gb::ceil_div(n, 256), 256>>>(n, b, e);
  GB_CUDA_TRY(cudaGetLastError());
  if (!weighted) {
    const double one_over_norme = 1. / sqrt((double)n);
    cuda_scal(n, one_over_norme, e);
    const double be = -cuda_dot(n, e, b);
    cuda_axpy(n, be, e, b);
  } else {
    double* aux = work;  // d, then sqrt(d); vec_vec(aux, e) with e = 1 leaves it unchanged
    gb::diagonal_kernel<<<gb::ceil_div(n, 256), 256>>>(n, ia, ja, a, aux);
    GB_CUDA_TRY(cudaGetLastError());
    cuda_vector_sqrt(n, aux, aux);
    double de_norm = cuda_dot(n, aux, aux);
    de_norm = 1.0 / sqrt(de_norm);
    cuda_scal(n, de_norm, aux);
    const double bwe = -cuda_dot(n, b, aux);
    cuda_axpy(n, bwe, aux, b);
  }
  GB_CUDA_TRY(cudaDeviceSynchronize());
  return GB_OK;
}

extern "C" int gb_synchronize(void) {
  GB_CUDA_TRY(cudaDeviceSynchronize());
  return GB_OK;
}
