// tri_plan.cu -- tiled record schedule of a triangular factor (replacing the
// csrsv2 analysis of cuda_blas.cu:99-224) and its launchers.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gb_common.cuh"
#include "kernels.h"
#include "sptrsv.h"
#include "tri_kernel.cuh"

namespace gb {

template <typename V>
static int upload(V** dst, const std::vector<V>& src) {
  const size_t bytes = sizeof(V) * std::max<size_t>(src.size(), 1);
  GB_CUDA_TRY(cudaMalloc(dst, bytes));
  if (!src.empty()) GB_CUDA_TRY(cudaMemcpy(*dst, src.data(), sizeof(V) * src.size(), cudaMemcpyHostToDevice));
  return GB_OK;
}

int tri_default_tile_rows(int n) {
  // GBLAP_TRI_TILE_ROWS overrides (32..16384; the autotuner's knob)
  if (const char* e = getenv("GBLAP_TRI_TILE_ROWS")) {
    const int v = atoi(e);
    if (v >= 32 && v <= kTriMaxTileRows64) return v;
  }
  // one tile per SM when the matrix is large; at least 1024 rows, at most
  // 16384 (128 KB of FP64 shared memory beside the 64 KB record ring)
  const int sms = device_sm_count();
  int t = 1024;
  while (t < 16384 && (long long)t * sms < n) t <<= 1;
  return t;
}

namespace {

// Rows with more dependencies get a LONG record.  A SHORT record holding a
// single row of kLongDeps dependencies must fit a ring slot:
// header + 4*4 + 2*8*4 + kLongDeps*4*12 <= kTriSlotBytes.
constexpr int kLongDeps = 32;
static_assert(kRecHdrBytes + 16 + 64 + kLongDeps * 4 * 12 <= kTriSlotBytes, "record slot too small");

// bytes of a SHORT record with `rows` rows of up to `len` dependencies
inline long long rec_size(int rows, int len, int S) {
  const long long R4 = (rows + 3) & ~3;
  return kRecHdrBytes + 4 * R4 + 2LL * S * R4 + (long long)len * R4 * (4 + S);
}

struct RecDesc {
  int wait_for;  // records of the tile in earlier levels (all must be done first)
  bool is_long;
  int len;
  std::vector<int> rows;
  int part = -1;  // split row: >= 0 the part's index, -2 the combine record
  int nparts = 0, slot0 = 0;
  int first = 0;  // a part: its first entry within the row
};

// Lays out all records in precision S; fills the RecordSet's host images.
// fixed (S = 4, short records only): the fixed layout of tri_kernel.cuh,
// with ddst = -1 (no diagonal slot) and vdsrc = each value's row diagonal.
void layout(const TriDeps& d, const std::vector<RecDesc>& recs, int S, std::vector<unsigned char>& buf,
            std::vector<long long>& off, std::vector<int>& nbytes, std::vector<long long>& vdst,
            std::vector<long long>& ddst, std::vector<long long>& idst,
            std::vector<int>* vsrc, std::vector<int>* dsrc, std::vector<int>* long_col,
            std::vector<int>* long_src, bool fixed = false, std::vector<int>* vdsrc = nullptr) {
  buf.clear();
  off.clear();
  nbytes.clear();
  int long_base = 0;  // the current long row's first entry in long_col
  vdst.clear();
  ddst.clear();
  idst.clear();
  for (const RecDesc& r : recs) {
    const int nrows = (int)r.rows.size();
    if (fixed) {
      const long long base = (long long)buf.size();
      const long long bytes = kFixHdrBytes + (long long)kFixLaneBytes * nrows;
      off.push_back(base);
      nbytes.push_back((int)bytes);
      buf.resize(base + bytes, 0);
      int* hdr = reinterpret_cast<int*>(buf.data() + base);
      hdr[0] = nrows;
      hdr[1] = r.wait_for;
      hdr[2] = (int)off.size() - 1;  // record index: the consumer checks the staged copy against it
      hdr[3] = kFixTag;
      for (int t = 0; t < nrows; ++t) {
        const int row = r.rows[t];
        const long long lb = base + kFixHdrBytes + (long long)kFixLaneBytes * t;
        int* w = reinterpret_cast<int*>(buf.data() + lb);
        w[0] = row;
        for (int k = 0; k < kTriHeld; ++k) w[1 + k] = -1;
        ddst.push_back(-1);
        idst.push_back(lb / 4 + 1 + kTriHeld);
        if (dsrc) dsrc->push_back(d.diag_src[row]);
        for (int k = d.row_ptr[row], e = 0; k < d.row_ptr[row + 1]; ++k, ++e) {
          w[1 + e] = d.dep_col[k];
          vdst.push_back(lb / 4 + 2 + kTriHeld + e);
          if (vsrc) vsrc->push_back(d.dep_src[k]);
          if (vdsrc) vdsrc->push_back(d.diag_src[row]);
        }
      }
      continue;
    }
    const long long R4 = (nrows + 3) & ~3;
    const long long bytes = r.is_long ? rec_size(nrows, 0, S) : rec_size(nrows, r.len, S);
    const long long base = (long long)buf.size();
    off.push_back(base);
    nbytes.push_back((int)bytes);
    buf.resize(base + bytes, 0);
    int* hdr = reinterpret_cast<int*>(buf.data() + base);
    hdr[0] = nrows;
    hdr[1] = r.len;
    hdr[2] = r.is_long ? kRecLong : 0;
    hdr[3] = 0;
    hdr[4] = r.wait_for;
    hdr[5] = (int)off.size() - 1;  // record index: the consumer checks the staged copy against it
    int* rows = hdr + kRecHdrBytes / 4;
    for (long long t = 0; t < R4; ++t) rows[t] = t < nrows ? r.rows[t] : -1;
    const long long diag_el = (base + kRecHdrBytes + 4 * R4) / S;  // element index of diag[0]
    for (int t = 0; t < nrows; ++t) {
      ddst.push_back(diag_el + t);
      idst.push_back(diag_el + R4 + t);
      if (dsrc) dsrc->push_back(d.diag_src[r.rows[t]]);
    }
    if (r.is_long) {
      const int row = r.rows[0];
      if (r.part == -2) {  // combine: parts and first slot
        hdr[1] = r.nparts;
        hdr[2] = kRecLong | kRecCombine;
        hdr[6] = r.slot0;
        continue;
      }
      if (r.part <= 0) {  // a whole long row, or its first part: the row's entries
        long_base = long_col ? (int)long_col->size() : 0;
        if (long_col)
          for (int k = d.row_ptr[row]; k < d.row_ptr[row + 1]; ++k) {
            long_col->push_back(d.dep_col[k]);
            long_src->push_back(d.dep_src[k]);
          }
      }
      hdr[3] = long_base + (r.part > 0 ? r.first : 0);
      if (r.part >= 0) {
        hdr[2] = kRecLong | kRecPart;
        hdr[6] = r.slot0 + r.part;
      }
      continue;
    }
    int* cols = reinterpret_cast<int*>(buf.data() + base + kRecHdrBytes + 4 * R4 + 2 * S * R4);
    const long long vals_el = (base + kRecHdrBytes + 4 * R4 + 2 * S * R4 + 4LL * r.len * R4) / S;
    for (long long q = 0; q < (long long)r.len * R4; ++q) cols[q] = -1;
    for (int t = 0; t < nrows; ++t) {
      const int row = r.rows[t];
      for (int k = d.row_ptr[row], e = 0; k < d.row_ptr[row + 1]; ++k, ++e) {
        cols[e * R4 + t] = d.dep_col[k];
        vdst.push_back(vals_el + e * R4 + t);
        if (vsrc) vsrc->push_back(d.dep_src[k]);
      }
    }
  }
}

int upload_set(RecordSet* rs, const std::vector<unsigned char>& buf, const std::vector<long long>& off,
               const std::vector<int>& nbytes, const std::vector<long long>& vdst,
               const std::vector<long long>& ddst, const std::vector<long long>& idst, size_t nlong,
               size_t S) {
  rs->bytes = (long long)buf.size();
  GB_TRY(upload(&rs->buf, buf));
  GB_TRY(upload(&rs->off, off));
  GB_TRY(upload(&rs->nbytes, nbytes));
  GB_TRY(upload(&rs->vdst, vdst));
  GB_TRY(upload(&rs->ddst, ddst));
  GB_TRY(upload(&rs->idst, idst));
  GB_CUDA_TRY(cudaMalloc(&rs->long_val, S * std::max<size_t>(nlong, 1)));
  return GB_OK;
}

void free_set(RecordSet* rs) {
  void* p[] = {rs->buf, rs->off, rs->nbytes, rs->vdst, rs->ddst, rs->idst, rs->long_val};
  for (void* q : p)
    if (q) cudaFree(q);
  *rs = RecordSet();
}

}  // namespace

int tri_plan_build(const TriDeps& d, TriPlan* plan, int tile_rows, int level_run) {
  const int n = d.n;
  const bool lower = d.lower;
  if (tile_rows <= 0) tile_rows = tri_default_tile_rows(n);
  tile_rows = std::max(32, std::min(tile_rows, kTriMaxTileRows32));
  auto deps_of = [&](int r) { return d.row_ptr[r + 1] - d.row_ptr[r]; };

  // global levels: the IC(0) factorization order and a diagnostic
  std::vector<int> lev(n, 0);
  int nlev = 0;
  for (int q = 0; q < n; ++q) {
    const int i = lower ? q : n - 1 - q;
    int l = 0;
    for (int k = d.row_ptr[i]; k < d.row_ptr[i + 1]; ++k) l = std::max(l, lev[d.dep_col[k]] + 1);
    lev[i] = l;
    nlev = std::max(nlev, l + 1);
  }
  std::vector<int> order;
  {
    std::vector<int> lptr(nlev + 1, 0);
    for (int i = 0; i < n; ++i) lptr[lev[i] + 1]++;
    for (int l = 0; l < nlev; ++l) lptr[l + 1] += lptr[l];
    std::vector<int> byl(n), fill(lptr.begin(), lptr.end() - 1);
    for (int i = 0; i < n; ++i) byl[fill[lev[i]]++] = i;
    for (int l = 0; l < nlev; ++l) {
      for (int p = lptr[l]; p < lptr[l + 1]; ++p) order.push_back(byl[p]);
      while (order.size() % 32) order.push_back(-1);
    }
  }

  // Form.  Contiguous row tiles keep a dependency inside the tile (shared
  // memory) when rows and their dependencies are near in index, as on grids.
  // When most dependencies cross tiles (a random labelling, power-law
  // graphs) the levels form takes over: records in global level order, cut
  // into runs of records (one per consumer warp) that CTAs take by ticket; with no
  // rows of their own, every dependency is read through L2.  Tiled, a tile
  // would wait on many earlier tiles, and tiles not yet resident start only
  // when whole earlier tiles have finished.  GBLAP_TRI_FORM=tiles|levels
  // forces a form.
  int nslots = 0;  // partial-sum slots of split hub rows
  bool levels_form = false;
  {
    long long cross = 0;
    for (int i = 0; i < n; ++i)
      for (int k = d.row_ptr[i]; k < d.row_ptr[i + 1]; ++k) cross += d.dep_col[k] / tile_rows != i / tile_rows;
    const long long total = (long long)d.dep_col.size();
    levels_form = total > 0 && 2 * cross > total;
    if (const char* e = getenv("GBLAP_TRI_FORM")) {
      if (!strcmp(e, "levels")) levels_form = true;
      if (!strcmp(e, "tiles")) levels_form = false;
    }
  }
  // entries per part of a split hub row; rows of more than two parts split
  int part_deps = kTriPartDeps;
  if (const char* e = getenv("GBLAP_TRI_PART_DEPS")) part_deps = std::max(32, atoi(e));
  const int ntiles = levels_form ? 0 : (n + tile_rows - 1) / tile_rows;
  std::vector<int> tr0, tr1, tile_rec{0}, rec_flags;
  std::vector<RecDesc> recs;
  std::vector<int> llev(levels_form ? 1 : tile_rows), bptr, bucket;
  int nlvl = 0;
  // rows of one level -> records (LONG rows alone, longest first; SHORT rows
  // packed up to kTriRecRows per record and the slot size)
  auto pack = [&](std::vector<int>& rows, int wait_for) {
    std::stable_sort(rows.begin(), rows.end(), [&](int a, int b) { return deps_of(a) > deps_of(b); });
    size_t p = 0;
    while (p < rows.size() && deps_of(rows[p]) > kLongDeps) {
      RecDesc r;
      r.wait_for = wait_for;
      r.is_long = true;
      r.len = deps_of(rows[p]);
      r.rows = {rows[p]};
      if (r.len > 2 * part_deps) {  // a hub: parts on any warps, then the combine
        const int np = (r.len + part_deps - 1) / part_deps;
        for (int k = 0; k < np; ++k) {
          RecDesc q = r;
          q.part = k;
          q.nparts = np;
          q.slot0 = nslots;
          q.first = k * part_deps;
          q.len = std::min(part_deps, r.len - k * part_deps);
          recs.push_back(q);
        }
        r.part = -2;
        r.nparts = np;
        r.slot0 = nslots;
        nslots += np;
      }
      recs.push_back(r);
      ++p;
    }
    while (p < rows.size()) {
      RecDesc r;
      r.wait_for = wait_for;
      r.is_long = false;
      r.len = deps_of(rows[p]);
      r.rows.push_back(rows[p++]);  // a SHORT row (<= kLongDeps deps) always fits a slot
      while (p < rows.size() && (int)r.rows.size() < kTriRecRows &&
             rec_size((int)r.rows.size() + 1, r.len, 8) <= kTriSlotBytes) {
        r.rows.push_back(rows[p]);
        ++p;
      }
      recs.push_back(r);
    }
  };
  if (levels_form) {
    std::vector<int> lptr(nlev + 1, 0), byl(n);
    for (int i = 0; i < n; ++i) lptr[lev[i] + 1]++;
    for (int l = 0; l < nlev; ++l) lptr[l + 1] += lptr[l];
    {
      std::vector<int> fill(lptr.begin(), lptr.end() - 1);
      for (int i = 0; i < n; ++i) byl[fill[lev[i]]++] = i;
    }
    for (int l = 0; l < nlev; ++l) {
      std::vector<int> rows(byl.begin() + lptr[l], byl.begin() + lptr[l + 1]);
      pack(rows, 0);  // no tile-local dependencies: nothing to wait for in the tile
    }
    // One record per consumer warp in each run: a level's records are
    // mostly independent, and a warp solves its records one after another,
    // so a run longer than the warps serialises a level on one CTA while
    // the other CTAs wait on it (4.19M-row Chung-Lu, FP32 lower solve:
    // 8.6 ms with runs of 128 records, 1.7 ms with 16).
    size_t run = level_run > 0 ? level_run : TriCons<double>::n;
    if (const char* e = getenv("GBLAP_TRI_LEVEL_RUN")) run = (size_t)std::max(1, atoi(e));
    for (size_t r0 = 0; r0 < recs.size(); r0 += run) {
      tr0.push_back(0);
      tr1.push_back(0);
      tile_rec.push_back((int)std::min(recs.size(), r0 + run));
    }
    nlvl = nlev;
  }
  for (int q = 0; q < ntiles; ++q) {
    const int tix = lower ? q : ntiles - 1 - q;
    const int t0 = tix * tile_rows, t1 = std::min(n, t0 + tile_rows);
    tr0.push_back(t0);
    tr1.push_back(t1);
    // Rows of the tile in GLOBAL level order.  A row's dependencies all have
    // lower global levels, so the in-tile ones sit in earlier buckets; and
    // where a tile splits the dependency structure (a 96^3 grid's 9216-row
    // planes in 8192-row tiles), a row's place in the tile also follows the
    // dependencies in other tiles, which levels counted inside the tile alone
    // would ignore -- those put rows that wait on a late other tile ahead of
    // rows that could run (20x slower at 96^3).  On aligned tiles the two
    // orders agree.
    int lmin = nlev, lmax = -1;
    for (int i = t0; i < t1; ++i) {
      lmin = std::min(lmin, lev[i]);
      lmax = std::max(lmax, lev[i]);
    }
    const int nl = lmax - lmin + 1;
    for (int i = t0; i < t1; ++i) llev[i - t0] = lev[i] - lmin;
    nlvl += nl;
    bptr.assign(nl + 1, 0);
    for (int i = t0; i < t1; ++i) bptr[llev[i - t0] + 1]++;
    for (int l = 0; l < nl; ++l) bptr[l + 1] += bptr[l];
    bucket.resize(t1 - t0);
    std::vector<int> fill(bptr.begin(), bptr.end() - 1);
    for (int i = t0; i < t1; ++i) bucket[fill[llev[i - t0]]++] = i;
    const size_t tile_first = recs.size();
    for (int l = 0; l < nl; ++l) {
      std::vector<int> rows(bucket.begin() + bptr[l], bucket.begin() + bptr[l + 1]);
      // longest first, so records group rows of similar length
      pack(rows, (int)(recs.size() - tile_first));  // waits for every earlier level of the tile
    }
    tile_rec.push_back((int)recs.size());
  }
  for (const RecDesc& r : recs) rec_flags.push_back(r.is_long ? kRecLong : 0);

  std::vector<unsigned char> buf;
  std::vector<long long> off, vdst, ddst, idst;
  std::vector<int> nbytes, vsrc, dsrc, long_col, long_src;
  layout(d, recs, 8, buf, off, nbytes, vdst, ddst, idst, &vsrc, &dsrc, &long_col, &long_src);
  for (int b : nbytes)  // every staged copy must fit its slot
    if (b <= 0 || b > kTriSlotBytes || (b & 15)) return GB_BAD_INPUT;
  plan->nval = (int)vsrc.size();
  plan->ndiag = (int)dsrc.size();
  plan->nlong = (int)long_col.size();
  GB_TRY(upload_set(&plan->r64, buf, off, nbytes, vdst, ddst, idst, long_col.size(), 8));
  plan->short_only = true;
  for (const RecDesc& r : recs)
    if (r.is_long || r.len > kTriHeld) plan->short_only = false;
  if (const char* e = getenv("GBLAP_TRI_SHORT"))  // 0: always the general kernel
    if (e[0] == '0') plan->short_only = false;
  // the FP32 records of a short-only plan in the fixed layout
  // (GBLAP_TRI_FIXED=0: the general layout)
  plan->fixed32 = plan->short_only;
  if (const char* e = getenv("GBLAP_TRI_FIXED"))
    if (e[0] == '0') plan->fixed32 = false;
  {
    // same record order, so the FP32 pass yields the same value/long order
    std::vector<int> vs2, ds2, lc2, ls2, vds;
    layout(d, recs, 4, buf, off, nbytes, vdst, ddst, idst, &vs2, &ds2, &lc2, &ls2, plan->fixed32,
           plan->fixed32 ? &vds : nullptr);
    if (plan->fixed32) GB_TRY(upload(&plan->vdsrc, vds));
  }
  GB_TRY(upload_set(&plan->r32, buf, off, nbytes, vdst, ddst, idst, long_col.size(), 4));
  plan->n = n;
  plan->lower = lower;
  plan->nlevels = nlev;
  plan->nslots = nslots;
  if (nslots > 0) {
    GB_CUDA_TRY(cudaMalloc(&plan->part64, sizeof(double) * nslots));
    GB_CUDA_TRY(cudaMalloc(&plan->part32, sizeof(float) * nslots));
    GB_TRY(fill_sentinel_dev(nslots, plan->part64, 0));
    GB_TRY(fill_sentinel_dev(nslots, plan->part32, 0));
    GB_CUDA_TRY(cudaDeviceSynchronize());
  }
  plan->tile_rows = levels_form ? 0 : tile_rows;
  plan->ntiles = (int)tr0.size();
  plan->levels_form = levels_form;
  plan->nlvl = nlvl;
  plan->nrec = (int)recs.size();
  plan->ndeps = (long long)d.dep_col.size();
  plan->norder = (int)order.size();
  GB_TRY(upload(&plan->tile_row0, tr0));
  GB_TRY(upload(&plan->tile_row1, tr1));
  GB_TRY(upload(&plan->tile_rec, tile_rec));
  GB_TRY(upload(&plan->rec_flags, rec_flags));
  GB_TRY(upload(&plan->vsrc, vsrc));
  GB_TRY(upload(&plan->dsrc, dsrc));
  GB_TRY(upload(&plan->long_col, long_col));
  GB_TRY(upload(&plan->long_src, long_src));
  GB_TRY(upload(&plan->order, order));
  GB_CUDA_TRY(cudaMalloc(&plan->ticket, sizeof(unsigned) * 4));
  GB_CUDA_TRY(cudaMemset(plan->ticket, 0, sizeof(unsigned) * 4));
  return GB_OK;
}

void tri_plan_free(TriPlan* p) {
  free_set(&p->r64);
  free_set(&p->r32);
  if (p->buf64s) cudaFree(p->buf64s);
  void* ptrs[] = {p->tile_row0, p->tile_row1, p->tile_rec, p->rec_flags, p->vsrc,   p->dsrc,  p->long_col,
                  p->long_src,  p->order,     p->ticket,   p->part64,    p->part32, p->vdsrc};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  *p = TriPlan();
}

// Writes the factor's values into the record buffers (FP64 and, when asked,
// FP32): entries, diagonals and their reciprocals, long-row values.
template <typename T>
__global__ void fill_records_kernel(int nval, const long long* __restrict__ vdst,
                                    const int* __restrict__ vsrc, const double* __restrict__ ent,
                                    int ndiag, const long long* __restrict__ ddst,
                                    const long long* __restrict__ idst, const int* __restrict__ dsrc,
                                    const double* __restrict__ dg, int nlong,
                                    const int* __restrict__ lsrc, T* buf, T* lval) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nval; i += stride) buf[vdst[i]] = (T)ent[vsrc[i]];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndiag; i += stride) {
    const double v = dg[dsrc[i]];
    if (ddst[i] >= 0) buf[ddst[i]] = (T)v;
    buf[idst[i]] = (T)(v != 0.0 ? 1.0 / v : 0.0);
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlong; i += stride) lval[i] = (T)ent[lsrc[i]];
}

// FP32 records in the fixed layout: the FMA form written directly -- each
// entry times its row's reciprocal diagonal in FP64, rounded once (the same
// values scale_records_kernel gives the general layout), and the
// reciprocals.
__global__ void fill_fixed32_kernel(int nval, const long long* __restrict__ vdst, const int* __restrict__ vsrc,
                                    const int* __restrict__ vdsrc, const double* __restrict__ ent, int ndiag,
                                    const long long* __restrict__ idst, const int* __restrict__ dsrc,
                                    const double* __restrict__ dg, float* buf) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nval; i += stride) {
    const double d = dg[vdsrc[i]];
    const double dinv = d != 0.0 ? 1.0 / d : 0.0;
    buf[vdst[i]] = (float)(ent[vsrc[i]] * dinv);
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndiag; i += stride) {
    const double d = dg[dsrc[i]];
    buf[idst[i]] = (float)(d != 0.0 ? 1.0 / d : 0.0);
  }
}

// FMA form: every short record's entry values times the reciprocal of their
// row's diagonal, computed in FP64 from the exact records and written to the
// FP64 copy (which already holds the rest of the record) and / or rounded
// once to the FP32 records (either may be null).  One warp per record, one
// lane per row.
__global__ void scale_records_kernel(int nrec, const long long* __restrict__ off64,
                                     const unsigned char* __restrict__ buf64,
                                     const long long* __restrict__ off32, unsigned char* buf32,
                                     unsigned char* buf64s) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int rec = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); rec < nrec; rec += warps) {
    const unsigned char* r = buf64 + off64[rec];
    const RecHdr h = *reinterpret_cast<const RecHdr*>(r);
    if ((h.flags & kRecLong) != 0 || lane >= h.nrows) continue;
    const int R4 = (h.nrows + 3) & ~3;
    const size_t vals64 = sizeof(RecHdr) + (size_t)R4 * (4 + 8 + 8) + (size_t)h.len * R4 * 4;
    const size_t vals32 = sizeof(RecHdr) + (size_t)R4 * (4 + 4 + 4) + (size_t)h.len * R4 * 4;
    const double dinv = reinterpret_cast<const double*>(r + sizeof(RecHdr) + (size_t)R4 * 12)[lane];
    const double* v = reinterpret_cast<const double*>(r + vals64);
    double* vs = buf64s ? reinterpret_cast<double*>(buf64s + off64[rec] + vals64) : nullptr;
    float* v32 = buf32 ? reinterpret_cast<float*>(buf32 + off32[rec] + vals32) : nullptr;
    for (int k = 0; k < h.len; ++k) {
      const double x = v[k * R4 + lane] * dinv;
      if (vs) vs[k * R4 + lane] = x;
      if (v32) v32[k * R4 + lane] = (float)x;
    }
  }
}

int tri_default_tile_rows32(int n) {
  // GBLAP_TRI_TILE_ROWS32 overrides (32..32768)
  if (const char* e = getenv("GBLAP_TRI_TILE_ROWS32")) {
    const int v = atoi(e);
    if (v >= 32 && v <= kTriMaxTileRows32) return v;
  }
  // as the FP64 tile: half the shared memory, the other half for the inbox
  return tri_default_tile_rows(n);
}

int tri_plan_fill(TriPlan* p, const double* ent_src, const double* diag_src, int mode,
                  cudaStream_t s) {
  const int g = std::max(1, std::min(device_sm_count() * 8, ceil_div(std::max(p->nval, p->ndiag), 256)));
  fill_records_kernel<double><<<g, 256, 0, s>>>(p->nval, p->r64.vdst, p->vsrc, ent_src, p->ndiag,
                                                p->r64.ddst, p->r64.idst, p->dsrc, diag_src,
                                                p->nlong, p->long_src, (double*)p->r64.buf,
                                                (double*)p->r64.long_val);
  GB_CUDA_TRY(cudaGetLastError());
  if (mode == kFillFma32) {
    if (p->fixed32)
      fill_fixed32_kernel<<<g, 256, 0, s>>>(p->nval, p->r32.vdst, p->vsrc, p->vdsrc, ent_src, p->ndiag,
                                            p->r32.idst, p->dsrc, diag_src, (float*)p->r32.buf);
    else
      fill_records_kernel<float><<<g, 256, 0, s>>>(p->nval, p->r32.vdst, p->vsrc, ent_src, p->ndiag,
                                                   p->r32.ddst, p->r32.idst, p->dsrc, diag_src,
                                                   p->nlong, p->long_src, (float*)p->r32.buf,
                                                   (float*)p->r32.long_val);
    GB_CUDA_TRY(cudaGetLastError());
    p->have32 = true;
  }
  if (mode == kFillFma64) {
    if (!p->buf64s) GB_CUDA_TRY(cudaMalloc(&p->buf64s, (size_t)p->r64.bytes));
    GB_CUDA_TRY(cudaMemcpyAsync(p->buf64s, p->r64.buf, (size_t)p->r64.bytes, cudaMemcpyDeviceToDevice, s));
  }
  if (mode != kFillExact && !(mode == kFillFma32 && p->fixed32)) {  // fixed FP32 records are written scaled
    if (p->nrec > 0) {
      const int gs = std::max(1, std::min(device_sm_count() * 8, ceil_div(p->nrec, 8)));
      scale_records_kernel<<<gs, 256, 0, s>>>(p->nrec, p->r64.off, p->r64.buf, p->r32.off,
                                              mode == kFillFma32 && !p->fixed32 ? p->r32.buf : nullptr,
                                              mode == kFillFma64 ? p->buf64s : nullptr);
      GB_CUDA_TRY(cudaGetLastError());
    }
  }
  return GB_OK;
}

// ------------------------------------------------------------ launching
static int g_tri_bps = 0;

int tri_blocks_per_sm() {
  if (g_tri_bps == 0) {
    const char* e = getenv("GBLAP_TRI_BLOCKS_PER_SM");
    const int v = e ? atoi(e) : 0;
    g_tri_bps = (v >= 1 && v <= 8) ? v : 1;
  }
  return g_tri_bps;
}

void tri_set_blocks_per_sm(int bps) { g_tri_bps = std::max(1, std::min(8, bps)); }

// FP32 solves in thread-block clusters (distributed-shared-memory hand-off
// between consecutive tiles): GBLAP_TRI_CLUSTER=0 selects the per-CTA form,
// 4 or 8 a cluster size; unset, the launcher chooses.
int tri_cluster_size() {
  static int v = -2;
  if (v == -2) {
    const char* e = getenv("GBLAP_TRI_CLUSTER");
    const int x = e ? atoi(e) : -1;
    v = (x == 0 || x == 4 || x == 8 || x == 16) ? x : -1;
  }
  return v;
}

bool tri_fp64_clusters() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("GBLAP_TRI_FP64_CLUSTER");
    v = e && atoi(e) == 0 ? 0 : 1;
  }
  return v != 0;
}

int tri_consumer_warps(int elem_bytes) { return elem_bytes == 8 ? TriCons<double>::n : TriCons<float>::n; }

int tri_grid(int ntiles) {
  return std::max(1, std::min(ntiles, device_sm_count() * tri_blocks_per_sm()));
}

template <typename T>
TriArgs<T> tri_args(const TriPlan& p, T* y, int* err, bool fma_form) {
  const RecordSet& rs = sizeof(T) == 8 ? p.r64 : p.r32;
  TriArgs<T> A;
  A.ntiles = p.ntiles;
  A.tile_row0 = p.tile_row0;
  A.tile_row1 = p.tile_row1;
  A.tile_rec = p.tile_rec;
  A.rec_off = rs.off;
  A.rec_bytes = rs.nbytes;
  A.recbuf = (sizeof(T) == 8 && fma_form) ? p.buf64s : rs.buf;
  A.long_col = p.long_col;
  A.long_val = (const T*)rs.long_val;
  A.y = y;
  A.ticket = p.ticket;
  A.err = err;
  A.tile_rows = p.tile_rows;
  if constexpr (sizeof(T) == 8) A.part = reinterpret_cast<T*>(p.part64);
  else A.part = reinterpret_cast<T*>(p.part32);
  A.poll = p.nlvl > 0 && 2 * p.nrec >= 3 * p.nlvl;  // at least 1.5 records per tile-level
  return A;
}
template TriArgs<double> tri_args<double>(const TriPlan&, double*, int*, bool);
template TriArgs<float> tri_args<float>(const TriPlan&, float*, int*, bool);

int tri_solve_plain(const TriPlan* p, const double* x, double* y, int* err, cudaStream_t s) {
  if (p->n <= 0) return GB_OK;
  GB_TRY(fill_sentinel_dev(p->n, y, s));
  OpPlain<double> op{x};
  return tri_launch<double, OpPlain<double>, true>(*p, tri_args<double>(*p, y, err, false), op, s);
}

}  // namespace gb
